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
//     before any stream capture;
//   * MC-Glauber and sqrt(T_A T_B) models only (the MC-KLN table would need
//     an allocation).
// It calls no cudaMalloc, cudaFree or allocating library routine.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "../../include/supermc.h"
#include "smc_kernels.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 24u << 20;
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

// Parameter derivation for this entry point (the same formulae the context
// uses): sigma_in from the PDG-96 Regge fits (src/Regge96.cpp:27-50), the
// nucleon width (src/GaussianNucleonsCal.cpp:34-54), sigma_gg by Newton
// iteration on a 38-point rule (src/GaussianNucleonsCal.cpp:130-163) and the
// Woods-Saxon table of src/Nucleus.cpp:58-148.
double na_sigma_in(double ecm) {
  double s = ecm * ecm;
  double sig = 22.0 * std::pow(s, 0.079) + 56.1 * std::pow(s, -0.46);
  double bel = 2.0 * 2.3 + 2.0 * 2.3 + 4.0 * std::pow(s, 0.0808) - 4.2;
  return sig - 0.0511 * sig * sig / bel;
}

double na_sigma_gg(double siginNN, double width) {
  static const double xp[19] = {
      4.078514790458e-2, 1.220840253379e-1, 2.025704538921e-1, 2.817088097902e-1, 3.589724404794e-1,
      4.338471694324e-1, 5.058347179279e-1, 5.744560210478e-1, 6.392544158297e-1, 6.997986803792e-1,
      7.556859037540e-1, 8.065441676053e-1, 8.520350219324e-1, 8.918557390046e-1, 9.257413320486e-1,
      9.534663309335e-1, 9.748463285902e-1, 9.897394542664e-1, 9.980499305357e-1};
  static const double wp[19] = {
      8.152502928039e-2, 8.098249377060e-2, 7.990103324353e-2, 7.828784465821e-2, 7.615366354845e-2,
      7.351269258474e-2, 7.038250706690e-2, 6.678393797914e-2, 6.274093339213e-2, 5.828039914700e-2,
      5.343201991033e-2, 4.822806186076e-2, 4.270315850467e-2, 3.689408159400e-2, 3.083950054518e-2,
      2.457973973823e-2, 1.815657770961e-2, 1.161344471647e-2, 5.002880749632e-3};
  double xg[38], wg[38];
  for (int k = 0; k < 19; k++) {
    xg[19 + k] = (1.0 * xp[k]) / 2.0 + 0.5;
    wg[19 + k] = (1.0 * wp[k]) / 2.0;
    xg[18 - k] = (1.0 * -xp[k]) / 2.0 + 0.5;
    wg[18 - k] = (1.0 * wp[k]) / 2.0;
  }
  double sigin = siginNN * 0.1, Bmax = 5.0 * width, sigeff = 10.0, prev;
  int guard = 0;
  do {
    prev = sigeff;
    double sum = 0.0, dN = 0.0;
    for (int ib = 0; ib < 38; ib++) {
      double b = xg[ib] * Bmax, db = wg[ib] * Bmax;
      double Tpp = std::exp(-b * b / (4. * width * width)) / (M_PI * (4. * width * width));
      sum += 2 * M_PI * b * db * (1.0 - std::exp(-sigeff * Tpp));
      dN += 2 * M_PI * b * db * Tpp * std::exp(-sigeff * Tpp);
    }
    sigeff -= (sum - sigin) / dN;
  } while (std::fabs(sigeff - prev) > 1e-4 && ++guard < 1000);
  return sigeff;
}

smc::NucleusDev na_nucleus(int A, int deformed, double R_ov, double a_ov, double dmin_ov) {
  smc::NucleusDev n{};
  n.A = A;
  n.deformed = deformed;
  double Ad = A;
  double rad = 1.12 * std::pow(Ad, 0.333333) - 0.86 / std::pow(Ad, 0.333333), dr = 0.54;
  if (A == 197) { rad = 6.42; dr = 0.45; }
  else if (A == 63) { rad = 4.28; dr = 0.5; }
  else if (A == 238) { rad = 6.86; dr = 0.44; }
  else if (A == 208) { rad = 6.67; dr = 0.44; }
  else if (A == 129) { rad = 5.36; dr = 0.590; }
  if (R_ov > 0) rad = R_ov;
  if (a_ov > 0) dr = a_ov;
  n.R = rad;
  n.a = dr;
  n.d_min = dmin_ov > 0 ? dmin_ov : 0.9;
  if (deformed) {
    if (A == 197) { n.beta2 = -0.13; n.beta4 = -0.03; }
    else if (A == 63) { n.beta2 = 0.162; n.beta4 = 0.006; }
    else if (A == 129) { n.beta2 = 0.162; n.beta4 = -0.003; }
    else if (A == 238) { n.beta2 = 0.28; n.beta4 = 0.093; }
  }
  n.rmax_cut = rad + 2.5;
  n.rw_max = 1.0 / (1.0 + std::exp(-rad / dr));
  return n;
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

  smc::DevParams P{};
  const double sigin = p.sigin_override > 0 ? p.sigin_override : na_sigma_in(p.ecm);
  double width;
  if (p.shape_of_nucleons == 1) width = std::sqrt(0.1 * sigin / M_PI) / 2.0;
  else if (p.shape_of_nucleons == 2) width = std::sqrt(0.1 * sigin / M_PI) / std::sqrt(8.0);
  else width = p.gauss_nucl_width;
  P.nx = (int)((p.maxx - (-p.maxx)) / p.dx + 0.1) + 1;
  P.ny = (int)((p.maxy - (-p.maxy)) / p.dy + 0.1) + 1;
  P.xmin = -p.maxx; P.ymin = -p.maxy; P.dx = p.dx; P.dy = p.dy;
  P.width = width; P.w2 = width * width; P.quark_width = p.quark_width;
  P.peak = 1 / (2 * M_PI * width * width);
  P.dsq = 0.1 * sigin / M_PI / 1;
  P.sigin = sigin;
  P.sigma_gg = na_sigma_gg(sigin, width);
  P.alpha = p.alpha; P.final_factor = p.final_factor;
  if (p.cc_fluctuation_model == 6) {   // Gamma weights, MCnucl.cpp:1271-1301
    const double eps = 1e-8, th = p.cc_fluctuation_gamma_theta;
    P.fluct = 1;
    P.fluct_k_part = (1 - p.alpha + eps) / 2. * (1. / th);
    P.fluct_th_part = 2. / (1 - p.alpha + eps) * th;
    P.fluct_k_coll = (p.alpha + eps) * (1. / th);
    P.fluct_th_coll = 1. / (p.alpha + eps) * th;
  }
  P.which_mc_model = p.which_mc_model; P.sub_model = p.sub_model;
  P.shape_of_nucleons = p.shape_of_nucleons; P.shape_of_entropy = p.shape_of_entropy;
  P.collision_criterion = p.collision_criterion;
  P.npmin = p.npmin; P.npmax = p.npmax; P.bmin = p.bmin; P.bmax = p.bmax;
  P.nuc[0] = na_nucleus(p.Aproj, p.proj_deformed, p.proj_R, p.proj_a, p.proj_d_min);
  P.nuc[1] = na_nucleus(p.Atarg, p.targ_deformed, p.targ_R, p.targ_a, p.targ_d_min);
  P.seed = p.seed;
  P.max_attempts = 1;
  P.max_coll = p.max_collisions > 0 ? p.max_collisions : 2048;
  P.max_src = 2 * (p.Aproj + p.Atarg) + P.max_coll;
  P.ecc_from = p.ecc_from_order; P.ecc_to = p.ecc_to_order;
  P.want_ta = P.want_tb = 0;
  P.n_planes = p.which_mc_model == 5 ? 1 : 2;
  const double d_max = p.shape_of_nucleons == 1 ? 2. * std::sqrt(P.dsq) : 5. * width;
  const double span = std::max(2 * d_max, 8 * std::max(width, p.quark_width));
  P.splat_mw = (int)(span / std::min(p.dx, p.dy)) + 3;

  // capacity of the fixed scratch
  const size_t recs_bytes = ((sizeof(smc::EventRec) * (size_t)n) + 255) / 256 * 256;
  if ((size_t)n > kNoAllocScratchBytes / sizeof(smc::Source) ||
      recs_bytes + sizeof(smc::Source) * (size_t)P.max_src * (size_t)n > kNoAllocScratchBytes)
    return SMC_ERR_SCRATCH_LIMIT;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SMC_ERR_NO_DEVICE;
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
