// C ABI: PairFLARE::compute (lammps_plugins/pair_flare.cpp:68-184) on
// LAMMPS-shaped arrays.
//
// The full neighbor list of the local atoms (ilist order) becomes the pair
// list of the B2 kernels with the pair style's filter rsq < rc^2; the same
// forward / contraction / adjoint kernels as the periodic path run on it.
// Pair forces are scattered with FP64 atomics to the central atom (+) and to
// the neighbor (-, local or ghost); the virial is ev_tally_xyz's
// sum over pairs of del (x) f with del = x_i - x_j.
#include <cublas_v2.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "b2_kernels.h"
#include "capi_state.h"
#include "common.cuh"
#include "gemm_tc.h"
#include "internal.h"

namespace fpp {

// Pair geometry from the explicit list: rel = x_j - x_i, r = |rel|.
__global__ void k_pairs_from_list(int inum, const int *__restrict__ ilist,
                                  const int *__restrict__ offset,
                                  const int *__restrict__ nbrs,
                                  const double *__restrict__ x,
                                  const int *__restrict__ type, int nall,
                                  int *__restrict__ nbr_i, int *__restrict__ nbr_s,
                                  dvec4 *__restrict__ rel, float4 *__restrict__ rel32,
                                  int *__restrict__ species_local,
                                  DeviceStatus *status) {
  const int ii = blockIdx.x;
  if (ii >= inum) return;
  const int i = ilist[ii];
  if (threadIdx.x == 0) species_local[ii] = type[i] - 1;
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  for (int p = offset[ii] + threadIdx.x; p < offset[ii + 1]; p += blockDim.x) {
    const int j = nbrs[p];
    if (j < 0 || j >= nall) {
      set_status(status, FPP_ERR_INVALID, 201, p);
      nbr_i[p] = ii;
      nbr_s[p] = 0;
      rel[p] = dvec4{1e300, 1e300, 0, 0};
      rel32[p] = make_float4(0, 0, 0, 0);
      continue;
    }
    const double dx = dsub(x[3 * j], xi), dy = dsub(x[3 * j + 1], yi),
                 dz = dsub(x[3 * j + 2], zi);
    const double r = __dsqrt_rn(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)));
    nbr_i[p] = ii;
    nbr_s[p] = type[j] - 1;
    rel[p] = dvec4{r, dx, dy, dz};
    rel32[p] = make_float4((float)dx, (float)dy, (float)dz, (float)r);
  }
}

template <typename T>
__global__ void k_pair_scatter(long long npairs, const int *__restrict__ ilist,
                               const int *__restrict__ nbr_i,
                               const int *__restrict__ nbrs,
                               const dvec4 *__restrict__ rel,
                               const T *__restrict__ pair_f, double *__restrict__ f,
                               double *__restrict__ virial) {
  __shared__ double sv[6][128];
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v[6] = {0, 0, 0, 0, 0, 0};
  if (p < npairs) {
    const double fx = (double)pair_f[4 * p], fy = (double)pair_f[4 * p + 1],
                 fz = (double)pair_f[4 * p + 2];
    if (fx != 0.0 || fy != 0.0 || fz != 0.0) {
      const int i = ilist[nbr_i[p]], j = nbrs[p];
      atomicAdd(&f[3 * i], fx);
      atomicAdd(&f[3 * i + 1], fy);
      atomicAdd(&f[3 * i + 2], fz);
      atomicAdd(&f[3 * j], -fx);
      atomicAdd(&f[3 * j + 1], -fy);
      atomicAdd(&f[3 * j + 2], -fz);
      const dvec4 r = rel[p];
      const double dx = -r.y, dy = -r.z, dz = -r.w;
      v[0] = dx * fx;
      v[1] = dy * fy;
      v[2] = dz * fz;
      v[3] = dx * fy;
      v[4] = dx * fz;
      v[5] = dy * fz;
    }
  }
  for (int k = 0; k < 6; k++) sv[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < 6; k++) sv[k][threadIdx.x] += sv[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 6) atomicAdd(&virial[threadIdx.x], sv[threadIdx.x][0]);
}

__global__ void k_energy_sum(int inum, const double *__restrict__ e, double *out) {
  __shared__ double sm[256];
  double a = 0;
  for (int i = threadIdx.x; i < inum; i += blockDim.x) a += e[i];
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sm[0];
}

int lammps_load(fpp_model *m, int32_t nlocal, int32_t nall, const double *x,
                const int32_t *type, int32_t inum, const int32_t *ilist,
                const int32_t *numneigh, const int32_t *neighbors, cudaStream_t st) {
  if (nall < nlocal || nlocal < 0 || inum < 0 || inum > nall)
    return fail(FPP_ERR_INVALID, "bad atom counts");
  if (inum > 0 && (!x || !type || !ilist || !numneigh))
    return fail(FPP_ERR_INVALID, "null argument");
  for (int k = 0; k < nall; k++)
    if (type[k] < 1 || type[k] > m->n_species)
      return fail(FPP_ERR_INVALID, "atom type outside 1..n_species");
  for (int ii = 0; ii < inum; ii++)
    if (ilist[ii] < 0 || ilist[ii] >= nall || numneigh[ii] < 0)
      return fail(FPP_ERR_INVALID, "bad ilist / numneigh");
  {
    long long total = 0;
    for (int ii = 0; ii < inum; ii++) total += numneigh[ii];
    if (total > 0 && !neighbors) return fail(FPP_ERR_INVALID, "null neighbor list");
    if (total >= (1ll << 31)) return fail(FPP_ERR_CAPACITY, "more than 2^31 pairs");
    for (long long p = 0; p < total; p++)
      if (neighbors[p] < 0 || neighbors[p] >= nall)
        return fail(FPP_ERR_INVALID, "neighbor index outside 0..nall-1");
  }
  // a pair style may be the process's first caller: no structure has
  // uploaded the kernels' constant tables yet
  FPP_TRY(ensure_tables(st));
  if (!m->lammps) m->lammps = new fpp_lammps_ws();
  fpp_lammps_ws &w = *m->lammps;
  fpp_structure *s = &w.s;
  StructureState &S = s->st;
  std::vector<int> off(inum + 1, 0);
  for (int ii = 0; ii < inum; ii++) off[ii + 1] = off[ii] + numneigh[ii];
  const int np = off[inum];
  S.noa = inum;
  S.n_pairs = np;
  S.species_host.resize(inum);
  for (int ii = 0; ii < inum; ii++) S.species_host[ii] = type[ilist[ii]] - 1;
  s->layout_species = -1;  // species can change between calls
  S.ci.volume = 1.0;
  FPP_TRY(w.d_x.reserve(sizeof(double) * 3 * std::max(nall, 1)));
  FPP_TRY(w.d_type.reserve(sizeof(int) * std::max(nall, 1)));
  FPP_TRY(w.d_ilist.reserve(sizeof(int) * std::max(inum, 1)));
  FPP_TRY(w.d_nbrs.reserve(sizeof(int) * std::max(np, 1)));
  FPP_TRY(S.nbr_offset.reserve(sizeof(int) * (inum + 1)));
  FPP_TRY(S.species.reserve(sizeof(int) * std::max(inum, 1)));
  const size_t npp = std::max(np, 1);
  FPP_TRY(S.nbr_i.reserve(sizeof(int) * npp));
  FPP_TRY(S.nbr_s.reserve(sizeof(int) * npp));
  FPP_TRY(S.nbr_rel.reserve(sizeof(dvec4) * npp));
  FPP_TRY(S.nbr_rel32.reserve(sizeof(float4) * npp));
  FPP_TRY(S.nbr_rev.reserve(sizeof(int) * npp));
  FPP_TRY(S.status.reserve(sizeof(DeviceStatus)));
  FPP_CUDA(cudaMemsetAsync(S.status.ptr, 0, sizeof(DeviceStatus), st));
  if (nall) {
    FPP_CUDA(cudaMemcpyAsync(w.d_x.ptr, x, sizeof(double) * 3 * nall, cudaMemcpyHostToDevice, st));
    FPP_CUDA(cudaMemcpyAsync(w.d_type.ptr, type, sizeof(int) * nall, cudaMemcpyHostToDevice, st));
  }
  if (inum) FPP_CUDA(cudaMemcpyAsync(w.d_ilist.ptr, ilist, sizeof(int) * inum, cudaMemcpyHostToDevice, st));
  if (np) FPP_CUDA(cudaMemcpyAsync(w.d_nbrs.ptr, neighbors, sizeof(int) * np, cudaMemcpyHostToDevice, st));
  FPP_CUDA(cudaMemcpyAsync(S.nbr_offset.ptr, off.data(), sizeof(int) * (inum + 1),
                           cudaMemcpyHostToDevice, st));
  if (inum) {
    k_pairs_from_list<<<inum, 64, 0, st>>>(inum, w.d_ilist.as<int>(), S.nbr_offset.as<int>(),
                                           w.d_nbrs.as<int>(), w.d_x.as<double>(),
                                           w.d_type.as<int>(), nall, S.nbr_i.as<int>(),
                                           S.nbr_s.as<int>(), S.nbr_rel.as<dvec4>(),
                                           S.nbr_rel32.as<float4>(), S.species.as<int>(),
                                           S.status.as<DeviceStatus>());
    FPP_CUDA(cudaGetLastError());
  }
  S.rel64_valid = true;  // the FP64 pair table comes from LAMMPS's arrays
  return FPP_OK;
}

}  // namespace fpp

using namespace fpp;

namespace fpp {

// Device bytes the pair style needs per listed atom with max_neigh
// neighbors (the buffers of mapped_core and of the pair list), the
// estimate that sizes the atom batches under a memory cap.
static double pair_bytes_per_atom(const fpp_model *m, int max_neigh, int precision) {
  const double sb = (double)m->args.n_species * m->args.N * m->args.H;
  const double ldp = (double)((m->n_d + 63) / 64 * 64);
  double per = 4.0 * (2 * sb + 2 * ldp) + 2.0 * 2 * ldp  // c, u, V, w; split operand
               + 8.0 * 8;                                // norms, energies, rows
  if (precision == FPP_PREC_FP64) per += 8.0 * (2 * sb + 3 * ldp);
  // per neighbor: FP64 and FP32 geometry, indices, pair forces, the list
  per += (double)max_neigh * (32 + 16 + 4 * 4 + 16 + 4 + (precision == FPP_PREC_FP64 ? 16 : 0));
  return per;
}

}  // namespace fpp

extern "C" int fpp_model_set_max_memory(fpp_model *m, double bytes) {
  if (!m) return fail(FPP_ERR_INVALID, "null model");
  if (!(bytes >= 0)) return fail(FPP_ERR_INVALID, "bytes must be >= 0");
  m->max_memory = bytes;
  return FPP_OK;
}

extern "C" int fpp_model_pair_batches(const fpp_model *m, int32_t *n_batches) {
  if (!m || !n_batches) return fail(FPP_ERR_INVALID, "null argument");
  *n_batches = m->last_pair_batches;
  return FPP_OK;
}

extern "C" int fpp_pair_compute(fpp_model *m, int32_t nlocal, int32_t nall,
                                const double *x, const int32_t *type, int32_t inum,
                                const int32_t *ilist, const int32_t *numneigh,
                                const int32_t *neighbors, int precision, double *f,
                                double *eng_vdwl, double *virial, double *eatom,
                                void *stream) {
  if (!m) return fail(FPP_ERR_INVALID, "null model");
  if (m->args.kind != kB2)
    return fail(FPP_ERR_UNSUPPORTED, "the pair style maps B2 models only (pair_flare.cpp)");
  if (inum > 0 && !f) return fail(FPP_ERR_INVALID, "null argument");
  if (m->beta_power == 0)
    return fail(FPP_ERR_INVALID, "mapped coefficients not set");
  if (precision != FPP_PREC_FP64 && precision != FPP_PREC_MIXED)
    return fail(FPP_ERR_INVALID, "bad precision");
  if (inum < 0 || (inum > 0 && (!ilist || !numneigh)))
    return fail(FPP_ERR_INVALID, "bad ilist / numneigh");
  cudaStream_t st = (cudaStream_t)stream;
  // Atom batches under the memory cap (pair_flare_kokkos.cpp:145-177): the
  // cap less the mapped coefficients, over the bytes per atom; as many
  // batches as needed, sizes differing by at most one atom, the first ones
  // the larger.  No cap (0): one batch.
  int n_batches = 1;
  if (m->max_memory > 0 && inum > 0) {
    int max_neigh = 0;
    for (int ii = 0; ii < inum; ii++) max_neigh = std::max(max_neigh, (int)numneigh[ii]);
    const double beta_mem = (double)m->n_species * m->n_d * m->n_d * 8.0;
    const double avail = m->max_memory - beta_mem;
    const double per = pair_bytes_per_atom(m, max_neigh, precision);
    const long long fit = avail > 0 ? (long long)(avail / per) : 0;
    if (fit < 1) return fail(FPP_ERR_CAPACITY, "Not enough memory for even a single atom!");
    const int approx = (int)std::min<long long>(fit, inum);
    n_batches = (inum + approx - 1) / approx;
  }
  const int base = inum / n_batches;
  int remainder = inum - n_batches * base;
  std::vector<long long> nb_off(inum + 1, 0);
  for (int ii = 0; ii < inum; ii++) nb_off[ii + 1] = nb_off[ii] + numneigh[ii];
  std::vector<double> hf(3 * (size_t)nall, 0.0);
  double vir_total[6] = {0, 0, 0, 0, 0, 0}, e_total = 0;
  std::vector<double> he;
  int start = 0;
  for (int b = 0; b < n_batches; b++) {
    const int bs = base + (remainder-- > 0 ? 1 : 0);
    const int32_t *nbrs_b = neighbors ? neighbors + nb_off[start] : nullptr;
    FPP_TRY(lammps_load(m, nlocal, nall, x, type, bs, ilist + start, numneigh + start, nbrs_b,
                        st));
    fpp_lammps_ws &w = *m->lammps;
    fpp_structure *s = &w.s;
    StructureState &S = s->st;
    const int np = (int)S.n_pairs;
    FPP_TRY(w.d_f.reserve(sizeof(double) * 3 * std::max(nall, 1)));
    FPP_TRY(w.d_vir.reserve(sizeof(double) * 8));
    FPP_TRY(w.d_e.reserve(sizeof(double) * 8));
    if (nall) FPP_CUDA(cudaMemsetAsync(w.d_f.ptr, 0, sizeof(double) * 3 * nall, st));
    FPP_CUDA(cudaMemsetAsync(w.d_vir.ptr, 0, sizeof(double) * 8, st));
    // same kernels as fpp_predict_mapped, with the pair style's strict filter
    FPP_TRY(mapped_core(m, s, precision, st, /*strict=*/1));
    if (np) {
      if (precision == FPP_PREC_FP64)
        k_pair_scatter<double><<<(np + 127) / 128, 128, 0, st>>>(
            np, w.d_ilist.as<int>(), S.nbr_i.as<int>(), w.d_nbrs.as<int>(),
            S.nbr_rel.as<dvec4>(), S.pair_f.as<double>(), w.d_f.as<double>(),
            w.d_vir.as<double>());
      else
        k_pair_scatter<float><<<(np + 127) / 128, 128, 0, st>>>(
            np, w.d_ilist.as<int>(), S.nbr_i.as<int>(), w.d_nbrs.as<int>(),
            S.nbr_rel.as<dvec4>(), S.pair_f.as<float>(), w.d_f.as<double>(),
            w.d_vir.as<double>());
      FPP_CUDA(cudaGetLastError());
    }
    if (bs) k_energy_sum<<<1, 256, 0, st>>>(bs, S.atom_e.as<double>(), w.d_e.as<double>());
    FPP_CUDA(cudaGetLastError());
    std::vector<double> bf(3 * (size_t)nall);
    he.assign(bs, 0.0);
    double vir[6] = {0, 0, 0, 0, 0, 0}, etot = 0;
    FPP_CUDA(cudaStreamSynchronize(st));
    FPP_TRY(check_status(S, st, "pair compute"));
    if (nall)
      FPP_CUDA(cudaMemcpy(bf.data(), w.d_f.ptr, sizeof(double) * 3 * nall,
                          cudaMemcpyDeviceToHost));
    if (bs) {
      FPP_CUDA(cudaMemcpy(he.data(), S.atom_e.ptr, sizeof(double) * bs, cudaMemcpyDeviceToHost));
      FPP_CUDA(cudaMemcpy(&etot, w.d_e.ptr, sizeof(double), cudaMemcpyDeviceToHost));
    }
    FPP_CUDA(cudaMemcpy(vir, w.d_vir.ptr, sizeof(vir), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < bf.size(); k++) hf[k] += bf[k];
    e_total += etot;
    for (int k = 0; k < 6; k++) vir_total[k] += vir[k];
    if (eatom)
      for (int ii = 0; ii < bs; ii++) eatom[ilist[start + ii]] += he[ii];
    start += bs;
  }
  for (size_t k = 0; k < hf.size(); k++) f[k] += hf[k];
  if (eng_vdwl) *eng_vdwl += e_total;
  if (virial)
    for (int k = 0; k < 6; k++) virial[k] += vir_total[k];
  m->last_pair_batches = n_batches;
  return FPP_OK;
}
