// smc_inject_noalloc: the injected-positions pipeline (pairing, density,
// eccentricities) for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- a host
// framework that owns every byte of device memory through its own pool, a
// real-time or capture-time code path that must not change the allocation
// state, or a plugin whose host forbids allocations after start-up.  Such a
// caller brings its own device buffers for the inputs and outputs; the
// intermediate data this pipeline needs between its two kernels (event
// records and splat sources) live in one file-scope device array of fixed
// size instead of in buffers a context would allocate.
//
// Limits and rules (also stated in include/supermc.h):
//   * the scratch array is kNoAllocScratchBytes (24 MiB); a call needs
//     64 + 64 * (2 (A + B) + max_collisions) bytes per event, with
//     max_collisions = 2048 unless the parameters set it; larger requests
//     are refused with SMC_ERR_SCRATCH_LIMIT;
//   * every call shares the array and it keeps the last call's contents; the
//     kernels overwrite every scratch byte they read, so nothing needs
//     clearing between calls -- but two calls whose work overlaps on the GPU
//     (different streams, or different host threads) race on it;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.  Under lazy module loading (the CUDA
//     default) that first call is also when the module loads and the 24 MiB
//     are committed on the device: make it before the caller's own pool
//     takes the device memory, or run with CUDA_MODULE_LOADING=EAGER;
//   * max_collisions defaults to 2048 per event here (the context's default
//     is 4096); an event with more binary collisions reports
//     SMC_ERR_CAPACITY in its d_status entry;
//   * MC-Glauber and sqrt(T_A T_B) models only (the MC-KLN table would need
//     an allocation).
// It calls no cudaMalloc, cudaFree or allocating library routine.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "../../include/supermc.h"
#include "smc_derive.h"
#include "smc_kernels.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 24u << 20;
// per-event collision capacity unless the parameters set one (the context
// default, 4096, would halve the events a call can take)
constexpr int kNoAllocMaxCollisions = 2048;
constexpr int kMaxDevices = 64;

// the scratch: event records followed by the splat sources
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (host code only sees a host-side stand-in under its name).
smc_status scratch_address(int dev, unsigned char **out) {
  if (dev < 0 || dev >= kMaxDevices) return SMC_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SMC_ERR_CUDA;
    g_addr[dev] = p;
  }
  *out = static_cast<unsigned char *>(g_addr[dev]);
  return SMC_OK;
}


}  // namespace

extern "C" smc_status smc_inject_noalloc(const smc_params *params, int n, const double *d_xy_proj,
                                         const double *d_xy_targ, const double *d_b, double *d_ecc, float *d_rho,
                                         int *d_status, void *cuda_stream) {
  if (!params || n < 0 || !d_xy_proj || !d_xy_targ || !d_ecc || !d_rho || !d_status) return SMC_ERR_ARGUMENT;
  const smc_params &p = *params;
  if (p.which_mc_model != 5 && p.which_mc_model != 7) return SMC_ERR_CONFIG;
  if (p.which_mc_model == 5 && p.sub_model != 1 && p.sub_model != 2) return SMC_ERR_CONFIG;
  if (p.shape_of_nucleons != 1 && p.shape_of_nucleons != 2 && p.shape_of_nucleons != 4) return SMC_ERR_CONFIG;
  if (p.shape_of_entropy != 1 && p.shape_of_entropy != 2) return SMC_ERR_CONFIG;
  if (p.collision_criterion != 1 && p.collision_criterion != 2) return SMC_ERR_CONFIG;
  if (p.Aproj < 1 || p.Atarg < 1 || p.Aproj > smc::kMaxA || p.Atarg > smc::kMaxA) return SMC_ERR_CONFIG;
  if (!(p.dx > 0) || !(p.dy > 0) || !(p.maxx > 0) || !(p.maxy > 0)) return SMC_ERR_CONFIG;
  if (p.ecc_from_order < 1 || p.ecc_to_order > 9 || p.ecc_from_order > p.ecc_to_order) return SMC_ERR_CONFIG;
  if (p.cc_fluctuation_model != 0 && p.cc_fluctuation_model != 6) return SMC_ERR_CONFIG;   // no per-cell NBD here
  if (p.cc_fluctuation_model == 6 && !(p.cc_fluctuation_gamma_theta > 0)) return SMC_ERR_CONFIG;
  if (n == 0) return SMC_OK;

  // the same derivation as the context's (smc_derive.h)
  smc::DevParams P{};
  smc_host::derive_common(p, P);
  P.max_attempts = 1;
  P.max_coll = p.max_collisions > 0 ? p.max_collisions : kNoAllocMaxCollisions;
  P.max_src = 2 * (p.Aproj + p.Atarg) + P.max_coll;
  P.want_ta = P.want_tb = 0;
  P.n_planes = p.which_mc_model == 5 ? 1 : 2;

  // capacity of the fixed scratch
  const size_t recs_bytes = ((sizeof(smc::EventRec) * (size_t)n) + 255) / 256 * 256;
  if ((size_t)n > kNoAllocScratchBytes / sizeof(smc::Source) ||
      recs_bytes + sizeof(smc::Source) * (size_t)P.max_src * (size_t)n > kNoAllocScratchBytes)
    return SMC_ERR_SCRATCH_LIMIT;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SMC_ERR_NO_DEVICE;
  // the splat's shared memory for this grid must fit the device (as the
  // context checks at creation)
  int smem_optin = 0;
  if (cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return SMC_ERR_CUDA;
  if (smc::grid_smem(P) > (size_t)smem_optin) return SMC_ERR_CONFIG;
  unsigned char *base = nullptr;
  smc_status s = scratch_address(dev, &base);
  if (s) return s;
  smc::EventRec *recs = reinterpret_cast<smc::EventRec *>(base);
  smc::Source *srcs = reinterpret_cast<smc::Source *>(base + recs_bytes);

  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SMC_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  const int grid1 = std::max(1, std::min(n, 4 * sms));
  const int grid2 = std::max(1, std::min(n, 2 * sms));
  if (smc::launch_sample_pair(P, 0, n, d_xy_proj, d_xy_targ, d_b, recs, srcs, nullptr, nullptr, grid1, st) !=
      cudaSuccess)
    return SMC_ERR_CUDA;
  if (smc::launch_grid(P, n, recs, srcs, d_rho, nullptr, nullptr, nullptr, d_ecc, d_status, grid2, st) !=
      cudaSuccess)
    return SMC_ERR_CUDA;
  return SMC_OK;
}
