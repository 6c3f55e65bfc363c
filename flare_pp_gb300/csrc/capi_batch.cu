// C ABI: mapped-beta prediction of a batch of uneven structures in one pass.
//
// The structures' atoms and neighbor lists are packed into one structure
// (atoms concatenated, each pair list shifted by its structure's atom and pair
// offsets, the FP64 pair table authoritative as for lists given from
// outside), so the forward pass, the contraction and the adjoint each run as
// one launch over every atom of the batch.  A segmented reduction then sums
// each structure's atom energies and pair virials (pair_f (x) r over its own
// pair range), and each stress is its virial over its own volume.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "capi_state.h"
#include "internal.h"

namespace fpp {

// One structure's neighbor data and its place in the packed structure.
struct BatchSrc {
  const int *nbr_i, *nbr_j, *nbr_s, *rev, *offset, *species;
  const dvec4 *rel;
  const float4 *rel32;
  int noa, atom_off;
  long long np, pair_off;
};

// blockIdx.y = structure; its pairs (shifted by its atom and pair offsets)
// and atoms are copied into the packed arrays.
__global__ void k_batch_pack(const BatchSrc *__restrict__ src, int *__restrict__ o_i,
                             int *__restrict__ o_j, int *__restrict__ o_s,
                             int *__restrict__ o_rev, dvec4 *__restrict__ o_rel,
                             float4 *__restrict__ o_rel32, int *__restrict__ o_offset,
                             int *__restrict__ o_species) {
  const BatchSrc b = src[blockIdx.y];
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < b.np; p += stride) {
    const long long q = b.pair_off + p;
    o_i[q] = b.nbr_i[p] + b.atom_off;
    o_j[q] = b.nbr_j[p] + b.atom_off;
    o_s[q] = b.nbr_s[p];
    o_rev[q] = b.rev[p] >= 0 ? (int)(b.rev[p] + b.pair_off) : -1;
    o_rel[q] = b.rel[p];
    o_rel32[q] = b.rel32[p];
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < b.noa; i += stride) {
    o_offset[b.atom_off + i] = b.offset[i] + (int)b.pair_off;
    o_species[b.atom_off + i] = b.species[i];
  }
}

// Per structure (a block each): out[10 s] = sum of its atom energies,
// out[10 s + 1 + 3a + b] = sum over its pairs of f_a r_b.  Fixed-order tree
// sums (deterministic).
template <typename T, typename R>
__global__ void __launch_bounds__(256)
k_batch_sums(const int *__restrict__ atom_off, const long long *__restrict__ pair_off,
             const double *__restrict__ atom_e, const T *__restrict__ pair_f,
             const R *__restrict__ rel, double *__restrict__ out) {
  __shared__ double sm[10][256];
  const int s = blockIdx.x, t = threadIdx.x;
  double v[10];
#pragma unroll
  for (int k = 0; k < 10; k++) v[k] = 0.0;
  for (int i = atom_off[s] + t; i < atom_off[s + 1]; i += blockDim.x) v[0] += atom_e[i];
  for (long long p = pair_off[s] + t; p < pair_off[s + 1]; p += blockDim.x) {
    const double f[3] = {(double)pair_f[4 * p], (double)pair_f[4 * p + 1],
                         (double)pair_f[4 * p + 2]};
    double r[3];
    if constexpr (sizeof(R) == sizeof(dvec4)) {
      const dvec4 d = reinterpret_cast<const dvec4 *>(rel)[p];
      r[0] = d.y;  // (r, x, y, z)
      r[1] = d.z;
      r[2] = d.w;
    } else {
      const float4 d = reinterpret_cast<const float4 *>(rel)[p];
      r[0] = d.x;  // (x, y, z, r)
      r[1] = d.y;
      r[2] = d.z;
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) v[1 + 3 * a + b] += f[a] * r[b];
  }
#pragma unroll
  for (int k = 0; k < 10; k++) sm[k][t] = v[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w)
#pragma unroll
      for (int k = 0; k < 10; k++) sm[k][t] += sm[k][t + w];
    __syncthreads();
  }
  if (t < 10) out[10 * s + t] = sm[t][0];
}

}  // namespace fpp

using namespace fpp;

extern "C" int fpp_predict_mapped_batched(fpp_model *m, fpp_structure *const *structures,
                                          int32_t n_structures, int precision,
                                          double *energies, double *forces, double *stresses,
                                          void *stream) {
  if (!m || (n_structures > 0 && !structures)) return fail(FPP_ERR_INVALID, "null argument");
  if (n_structures < 0) return fail(FPP_ERR_INVALID, "negative structure count");
  if (n_structures == 0) return FPP_OK;
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<int> aoff(n_structures + 1, 0);
  std::vector<long long> poff(n_structures + 1, 0);
  for (int k = 0; k < n_structures; k++) {
    fpp_structure *s = structures[k];
    if (!s) return fail(FPP_ERR_INVALID, "null structure");
    FPP_TRY(ensure_rel64(s->st, st));  // the FP64 pair table of each list
    aoff[k + 1] = aoff[k] + s->st.noa;
    poff[k + 1] = poff[k] + s->st.n_pairs;
  }
  const int N = aoff[n_structures];
  const long long P = poff[n_structures];
  if (P >= (1ll << 31)) return fail(FPP_ERR_CAPACITY, "more than 2^31 pairs in the batch");
  if (!m->batch) m->batch = new fpp_structure();
  fpp_structure *b = m->batch;
  StructureState &B = b->st;
  B.noa = N;
  B.n_pairs = P;
  B.species_host.clear();
  for (int k = 0; k < n_structures; k++)
    B.species_host.insert(B.species_host.end(), structures[k]->st.species_host.begin(),
                          structures[k]->st.species_host.end());
  b->layout_species = -1;  // species differ from batch to batch
  B.ci.volume = 1.0;
  B.rel64_valid = true;    // the packed FP64 table is authoritative (cells differ)
  const size_t np = (size_t)std::max<long long>(P, 1);
  FPP_TRY(B.species.reserve(sizeof(int) * std::max(N, 1)));
  FPP_TRY(B.nbr_offset.reserve(sizeof(int) * (N + 1)));
  FPP_TRY(B.nbr_i.reserve(sizeof(int) * np));
  FPP_TRY(B.nbr_j.reserve(sizeof(int) * np));
  FPP_TRY(B.nbr_s.reserve(sizeof(int) * np));
  FPP_TRY(B.nbr_rev.reserve(sizeof(int) * np));
  FPP_TRY(B.nbr_rel.reserve(sizeof(dvec4) * np));
  FPP_TRY(B.nbr_rel32.reserve(sizeof(float4) * np));
  if (B.status.bytes < sizeof(DeviceStatus)) {
    FPP_TRY(B.status.reserve(sizeof(DeviceStatus)));
    FPP_CUDA(cudaMemsetAsync(B.status.ptr, 0, sizeof(DeviceStatus), st));
  }
  std::vector<BatchSrc> src(n_structures);
  long long max_work = 1;
  for (int k = 0; k < n_structures; k++) {
    StructureState &S = structures[k]->st;
    BatchSrc &q = src[k];
    q.nbr_i = S.nbr_i.as<int>();
    q.nbr_j = S.nbr_j.as<int>();
    q.nbr_s = S.nbr_s.as<int>();
    q.rev = S.nbr_rev.as<int>();
    q.offset = S.nbr_offset.as<int>();
    q.species = S.species.as<int>();
    q.rel = S.nbr_rel.as<dvec4>();
    q.rel32 = S.nbr_rel32.as<float4>();
    q.noa = S.noa;
    q.atom_off = aoff[k];
    q.np = S.n_pairs;
    q.pair_off = poff[k];
    max_work = std::max(max_work, std::max<long long>(S.n_pairs, S.noa));
  }
  FPP_TRY(m->batch_src.reserve(sizeof(BatchSrc) * n_structures));
  FPP_CUDA(cudaMemcpyAsync(m->batch_src.ptr, src.data(), sizeof(BatchSrc) * n_structures,
                           cudaMemcpyHostToDevice, st));
  const int tb = 256;
  const int bx = (int)std::min<long long>((max_work + tb - 1) / tb, 1024);
  for (int c0 = 0; c0 < n_structures; c0 += 65535) {  // grid y holds 65535 structures
    const int cy = std::min(65535, n_structures - c0);
    k_batch_pack<<<dim3(bx, cy), tb, 0, st>>>(
        m->batch_src.as<BatchSrc>() + c0, B.nbr_i.as<int>(), B.nbr_j.as<int>(),
        B.nbr_s.as<int>(), B.nbr_rev.as<int>(), B.nbr_rel.as<dvec4>(),
        B.nbr_rel32.as<float4>(), B.nbr_offset.as<int>(), B.species.as<int>());
    FPP_CUDA(cudaGetLastError());
  }
  const int P32 = (int)P;
  FPP_CUDA(cudaMemcpyAsync(B.nbr_offset.as<int>() + N, &P32, sizeof(int),
                           cudaMemcpyHostToDevice, st));
  FPP_TRY(mapped_core(m, b, precision, st, 0));
  // per-structure energies and virials
  DevBuf &d_aoff = m->batch_aoff, &d_poff = m->batch_poff, &d_out = m->batch_sums;
  FPP_TRY(d_aoff.reserve(sizeof(int) * (n_structures + 1)));
  FPP_TRY(d_poff.reserve(sizeof(long long) * (n_structures + 1)));
  FPP_TRY(d_out.reserve(sizeof(double) * 10 * n_structures));
  FPP_CUDA(cudaMemcpyAsync(d_aoff.ptr, aoff.data(), sizeof(int) * (n_structures + 1),
                           cudaMemcpyHostToDevice, st));
  FPP_CUDA(cudaMemcpyAsync(d_poff.ptr, poff.data(), sizeof(long long) * (n_structures + 1),
                           cudaMemcpyHostToDevice, st));
  if (precision == FPP_PREC_FP64)
    k_batch_sums<double, dvec4><<<n_structures, 256, 0, st>>>(
        d_aoff.as<int>(), d_poff.as<long long>(), B.atom_e.as<double>(),
        B.pair_f.as<double>(), B.nbr_rel.as<dvec4>(), d_out.as<double>());
  else
    k_batch_sums<float, float4><<<n_structures, 256, 0, st>>>(
        d_aoff.as<int>(), d_poff.as<long long>(), B.atom_e.as<double>(),
        B.pair_f.as<float>(), B.nbr_rel32.as<float4>(), d_out.as<double>());
  FPP_CUDA(cudaGetLastError());
  std::vector<double> sums(10 * (size_t)n_structures);
  DeviceStatus hs;
  FPP_CUDA(cudaMemcpyAsync(sums.data(), d_out.ptr, sizeof(double) * sums.size(),
                           cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaMemcpyAsync(&hs, B.status.ptr, sizeof(hs), cudaMemcpyDeviceToHost, st));
  if (forces && N)
    FPP_CUDA(cudaMemcpyAsync(forces, B.forces.ptr, sizeof(double) * 3 * N,
                             cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  if (hs.code != 0) {
    FPP_CUDA(cudaMemsetAsync(B.status.ptr, 0, sizeof(DeviceStatus), st));
    return fail(hs.code, "batched prediction: device status " + std::to_string(hs.code) +
                             " at " + std::to_string(hs.where));
  }
  for (int k = 0; k < n_structures; k++) {
    const double *r = sums.data() + 10 * (size_t)k;
    if (energies) energies[k] = r[0];
    if (stresses) {
      // -(1/V) sum f_a r_b, order xx xy xz yy yz zz
      const double vi = 1.0 / structures[k]->st.ci.volume;
      const int ab[6] = {0, 1, 2, 4, 5, 8};
      for (int c = 0; c < 6; c++) stresses[6 * k + c] = -r[1 + ab[c]] * vi;
    }
  }
  return FPP_OK;
}
