// C ABI: B2 descriptors without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need
// descriptors: an MD engine that owns all device memory through its own pool
// (nothing may be cudaMalloc'd behind its back), or a real-time loop with a
// fixed memory budget decided up front.  fpp_b2_descriptors_noalloc serves
// them: the caller passes the pair geometry and the output buffers, and the
// only scratch the forward kernel needs (the single-bond coefficients, an
// identity row map and the radial-pair table) lives in the fixed arrays below,
// which every GPU that loads this library holds until the process exits.
//
// The first call on a device does a one-time set-up with that device current:
// it resolves the arrays' device addresses (cudaGetSymbolAddress), uploads the
// harmonic normalisation table and synchronizes the stream.  Make that first
// call before any stream capture begins.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "b2_kernels.h"
#include "capi_state.h"
#include "common.cuh"
#include "internal.h"

namespace fpp {

// Scratch limits: n_atoms * n_species * N * (lmax+1)^2 <= kNoAllocC doubles
// (8 MiB) and n_atoms <= kNoAllocAtoms.
constexpr size_t kNoAllocC = 1u << 20;
constexpr int kNoAllocAtoms = 1 << 16;
constexpr int kNoAllocPairTab = 64 * 65 / 2;  // n_rad <= 64

static __device__ __align__(256) double g_noalloc_c[kNoAllocC];
static __device__ __align__(256) int g_noalloc_rows[kNoAllocAtoms];
static __device__ __align__(256) int g_noalloc_tab[kNoAllocPairTab];

// Device addresses of the arrays above, resolved once per device.  In host
// code the arrays' names stand for host-side shadows, never device addresses.
struct NoAllocSlot {
  std::atomic<bool> ready{false};
  double *c = nullptr;
  int *rows = nullptr;
  int *tab = nullptr;
};
static NoAllocSlot g_slots[64];
static std::mutex g_setup_mu;  // serialises first calls from several host threads

static int noalloc_setup(NoAllocSlot **out, cudaStream_t st) {
  int dev = 0;
  FPP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FPP_ERR_UNSUPPORTED, "device index beyond 63");
  NoAllocSlot &s = g_slots[dev];
  if (!s.ready.load(std::memory_order_acquire)) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!s.ready.load(std::memory_order_relaxed)) {
      FPP_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.c), g_noalloc_c));
      FPP_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.rows), g_noalloc_rows));
      FPP_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.tab), g_noalloc_tab));
      if (upload_harmonic_tables(st) != 0)
        return fail(FPP_ERR_CUDA, "upload of harmonic tables failed");
      FPP_CUDA(cudaStreamSynchronize(st));
      // the addresses above become visible to other threads with the flag
      s.ready.store(true, std::memory_order_release);
    }
  }
  *out = &s;
  return FPP_OK;
}

// Identity row map and the (n1, n2 >= n1) radial-pair table, rewritten on
// every call (the arrays keep the previous call's contents).
__global__ void k_noalloc_tables(int n_atoms, int nr, int *__restrict__ rows,
                                 int *__restrict__ tab) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_atoms) rows[t] = t;
  const int npair = nr * (nr + 1) / 2;
  if (t < npair) {
    int n1 = 0, q = t;
    while (q >= nr - n1) {
      q -= nr - n1;
      n1++;
    }
    tab[t] = n1 | ((n1 + q) << 16);
  }
}

}  // namespace fpp

using namespace fpp;

extern "C" int fpp_b2_descriptors_noalloc(const fpp_b2 *b2, int32_t n_atoms,
                                          const int32_t *species, const int32_t *offsets,
                                          const double *rel, const int32_t *nbr_species,
                                          double *descriptors, double *norms,
                                          void *stream) {
  if (!b2) return fail(FPP_ERR_INVALID, "null descriptor");
  if (n_atoms < 0) return fail(FPP_ERR_INVALID, "n_atoms < 0");
  if (n_atoms == 0) return FPP_OK;
  if (!species || !offsets || !rel || !nbr_species || !descriptors || !norms)
    return fail(FPP_ERR_INVALID, "null argument");
  const B2Args &a0 = b2->args;
  if (a0.kind != kB2)
    return fail(FPP_ERR_UNSUPPORTED, "fpp_b2_descriptors_noalloc computes B2 descriptors only");
  const int nr = a0.n_species * a0.N;
  const size_t sb = (size_t)nr * a0.H;
  if (n_atoms > kNoAllocAtoms || (size_t)n_atoms * sb > kNoAllocC)
    return fail(FPP_ERR_CAPACITY,
                "fpp_b2_descriptors_noalloc handles at most " +
                    std::to_string(kNoAllocC / sb < (size_t)kNoAllocAtoms ? kNoAllocC / sb
                                                                        : (size_t)kNoAllocAtoms) +
                    " atoms for this descriptor (scratch of 8 MiB)");
  if (nr * (nr + 1) / 2 > kNoAllocPairTab)
    return fail(FPP_ERR_CAPACITY, "n_species * N above 64");
  if (reinterpret_cast<uintptr_t>(rel) % 32 != 0)
    return fail(FPP_ERR_INVALID, "rel must be 32-byte aligned (n_pairs x 4 doubles)");
  cudaStream_t st = (cudaStream_t)stream;
  NoAllocSlot *slot = nullptr;
  FPP_TRY(noalloc_setup(&slot, st));
  const int nt = n_atoms > nr * (nr + 1) / 2 ? n_atoms : nr * (nr + 1) / 2;
  k_noalloc_tables<<<ceil_div(nt, 256), 256, 0, st>>>(n_atoms, nr, slot->rows, slot->tab);
  FPP_CUDA(cudaGetLastError());
  B2Args a = a0;
  a.noa = n_atoms;
  a.strict = 0;
  Neigh nb;
  std::memset(&nb, 0, sizeof(nb));  // geom.wp == nullptr: rel is the FP64 table
  nb.offset = offsets;
  nb.rel = reinterpret_cast<const dvec4 *>(rel);
  nb.rel32 = nullptr;  // read only by the FP32 instantiation
  nb.nbr_s = nbr_species;
  nb.rev = nullptr;
  if (launch_b2_forward<double>(a, nb, species, slot->rows, slot->tab, slot->c, descriptors,
                                norms, nullptr, nullptr, nullptr, 0, nullptr, st) != 0)
    return fail(FPP_ERR_CUDA, "B2 forward (no-allocation) launch failed");
  return FPP_OK;
}
