// Host runtime behind the C ABI of include/supermc.h: configuration and
// derived constants (MCnucl::MCnucl, src/MCnucl.cpp:22-154), device buffers,
// batching and the two-stage launch sequence.
#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <vector>

#include "../../include/supermc.h"
#include "smc_derive.h"
#include "smc_kernels.h"

namespace {

using smc_host::derive_common;
using smc_host::make_nucleus;
using smc_host::sigma_gg_from;
using smc_host::sigma_inelastic;

using smc::DevParams;
using smc::EventRec;
using smc::Source;

// Gauss-Legendre rule on [0,1] (Newton iteration on P_n from the
// asymptotic initial guess).
void gauss_legendre01(int n, std::vector<double> &x, std::vector<double> &w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = 0.0;
      for (int j = 1; j <= n; j++) {
        double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p2) / j;
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p0 / dp;
      if (std::fabs(z - z1) < 1e-15) break;
    }
    x[i] = 0.5 * (1.0 - z);
    x[n - 1 - i] = 0.5 * (1.0 + z);
    w[i] = w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Inverse-CDF table of the Woods-Saxon radius (differentiable sampling
// mode): N, dN/dR, dN/da of int_0^r t^2 rho(t) dt, rho = 1/(1+exp((t-R)/a)),
// at r_k = k h on [0, R + 2.5], each step integrated by the 5-point
// Gauss-Legendre rule (published nodes and weights).
void icdf_table(smc::NucleusDev &n, std::vector<double> &tab) {
  const int m = 2048;
  const double rmax = n.R + 2.5, h = rmax / (m - 1);
  static const double x5[3] = {0.0, 0.5384693101056831, 0.9061798459386640};
  static const double w5[3] = {0.5688888888888889, 0.4786286704993665, 0.2369268850561891};
  auto integrand = [&](double t, double &f, double &fR, double &fa) {
    const double rho = 1.0 / (1.0 + std::exp((t - n.R) / n.a)), d = rho * (1.0 - rho) / n.a;
    f = t * t * rho;
    fR = t * t * d;
    fa = fR * (t - n.R) / n.a;
  };
  tab.assign((size_t)3 * m, 0.0);
  for (int k = 1; k < m; k++) {
    const double c = (k - 0.5) * h, hh = 0.5 * h;
    double s0 = 0, s1 = 0, s2 = 0;
    for (int q = 0; q < 3; q++)
      for (int sg = -1; sg <= (q == 0 ? -1 : 1); sg += 2) {
        double f, fR, fa;
        integrand(c + sg * hh * x5[q], f, fR, fa);
        s0 += w5[q] * hh * f;
        s1 += w5[q] * hh * fR;
        s2 += w5[q] * hh * fa;
      }
    tab[k] = tab[k - 1] + s0;
    tab[m + k] = tab[m + k - 1] + s1;
    tab[2 * m + k] = tab[2 * m + k - 1] + s2;
  }
  double f, fR, fa;
  integrand(rmax, f, fR, fa);
  // search starts: the largest node below each of nb + 1 evenly spaced fractions
  const int nb = 512;
  tab.resize((size_t)3 * m + nb + 1);
  for (int b = 0, k = 0; b <= nb; b++) {
    const double target = (double)b / nb * tab[m - 1];
    while (k + 1 < m && tab[k + 1] <= target) k++;
    tab[(size_t)3 * m + b] = k;
  }
  n.icdf_nb = nb;
  n.icdf_m = m;
  n.icdf_h = h;
  n.icdf_ntot = tab[m - 1];
  n.icdf_dntot_R = tab[2 * m - 1] + f;   // the end point rmax = R + 2.5 moves with R
  n.icdf_dntot_a = tab[3 * m - 1];
}

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t want) {
    if (want <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * want);
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

struct Ctx {
  smc_params prm{};
  DevParams P{};
  smc_info info{};
  int device = 0, sms = 0, dev_smem = 0;
  cudaStream_t own = nullptr, st = nullptr;
  int occ1 = 1, occ2 = 1;
  bool use_tc = true;   // tensor-core splat for the batched paths (when the profile allows it)
  int chunk = 4096;
  DevBuf<EventRec> recs;
  DevBuf<Source> srcs;
  DevBuf<double> ecc, pos, bvec, inj_p, inj_t, inj_b, coll;
  DevBuf<float> rho, ta, tb, scratch;
  DevBuf<int> status, npart, ncoll, attempts;
  // buffers of the tensor-core splat: per-event densities (when not an
  // output), per-CTA corner corrections, per-event centre-of-mass sums
  DevBuf<float> rho_ev;
  // event queues of the batched kernels: per-chunk order (most sources
  // first) and the tickets of the splat, moments and sampler launches
  DevBuf<int> ev_order, tickets;
  DevBuf<int> corr_ev;
  DevBuf<double> cm_ev;
  // mixed batches: system table, per-event system of the chunk, event order
  bool mixing = false;
  DevBuf<smc::SystemDev> mix_sys;
  DevBuf<int> mix_ev, mix_order;
  DevBuf<uint8_t> wounded;
  DevBuf<double> kln64;
  DevBuf<float> kln32;
  DevBuf<float4> kln_coef;
  // p_T-differential table (smc_kln_pt_table) [tmax][tmax][pt_nbins], its
  // bins, and the per-event thickness and p_T-differential staging buffers
  DevBuf<double> pt64;
  DevBuf<float> pt32, pt_ta, pt_tb, rho_pt;
  // staging of the per-event binary-collision and spectator densities
  DevBuf<float> ev_aux;
  int pt_nbins = 0;
  double pt_min = 0, pt_step = 0;
  // adjoint: forward densities, per-CTA adjoint grids, staged cotangents,
  // per-event gradients
  DevBuf<float> adj_rho, adj_lam, adj_grho;
  DevBuf<double> adj_geps, adj_out;
  // position tangents (differentiable sampling): inverse-CDF tables, the
  // per-nucleon and per-source tangents, injected tangents, and the set the
  // next sampler launch uses
  DevBuf<double> icdf_tab[2], ntan, inj_tp, inj_tt, orient;
  DevBuf<float4> stan;
  // light-nucleus configuration tables by mass number: [n][A][3] on the device
  struct ConfTab {
    DevBuf<double> xyz;
    int n = 0;
  };
  std::map<int, ConfTab> conf;
  smc::TangentIO tio{};
  std::vector<double> h_adj;
  // captured batch (smc_generate_graph): the instantiated graph and what it
  // was captured for, the device event-id base and worst status, and their
  // pinned host copies
  cudaGraphExec_t graph = nullptr;
  int graph_n = 0, graph_chunk = 0, graph_launches = 0;
  bool graph_tc = false;
  smc_outputs graph_out{};
  // the context's device buffers a captured batch uses (a buffer that a
  // later eager call had to grow is reallocated: the graph is captured again)
  std::array<const void *, 12> graph_bufs{}, mgraph_bufs{};
  // captured mixed-system batch (smc_generate_mixed_graph): its system table,
  // per-event systems and event order on the device, and what it was
  // captured for
  cudaGraphExec_t mgraph = nullptr;
  int mgraph_n = 0, mgraph_chunk = 0, mgraph_launches = 0;
  bool mgraph_tc = false;
  smc_outputs mgraph_out{};
  std::vector<smc_params> mgraph_sys;
  std::vector<int> mgraph_ev;
  DevBuf<smc::SystemDev> mg_sys;
  DevBuf<int> mg_ev, mg_order;
  DevBuf<uint64_t> ev_base;
  DevBuf<int> worst;
  uint64_t *h_first = nullptr;
  int *h_worst = nullptr;
  DevBuf<smc::AvgSrc> avg_state;
  // binned averages: event frames, bin order, bin segments and counts,
  // bin edges, per-bin compensated sums
  DevBuf<smc::AvgFrame> avg_frame;
  DevBuf<int> avg_order, avg_seg, avg_count, avg_edges;
  DevBuf<float2> avg_bins;
  DevBuf<float2> avg_part;   // per-slice bin sums of a chunk (smc_average_binned)
  DevBuf<float> avg_rho, avg_ta, avg_tb, avg_aux;
  DevBuf<Source> avg_view;
  DevBuf<EventRec> avg_vrecs;   // the view's records (every record may splat)
  DevBuf<int> avg_status;
  DevBuf<double> avg_acc;
  std::vector<int> h_status;
  std::vector<EventRec> h_recs;
  // counters and optional kernel timing
  smc_stats stats{};
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;   // kind, (start, stop)
  size_t ev_next = 0;
};

cudaEvent_t next_event(Ctx *c) {
  if (c->ev_next == c->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    c->ev_pool.push_back(e);
  }
  return c->ev_pool[c->ev_next++];
}

// brackets one kernel launch with events when timing is on
template <typename F>
cudaError_t timed(Ctx *c, int kind, F &&launch) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (c->timing) {
    a = next_event(c);
    b = next_event(c);
    if (a) cudaEventRecord(a, c->st);
  }
  cudaError_t e = launch();
  if (c->timing && a && b) {
    cudaEventRecord(b, c->st);
    c->pending.push_back({kind, {a, b}});
  }
  c->stats.launches++;
  if (kind == 0) c->stats.sample_launches++;
  else if (kind == 1) c->stats.grid_launches++;
  else c->stats.post_launches++;
  return e;
}

// folds recorded kernel durations into the counters (after a stream sync)
void collect_timing(Ctx *c) {
  for (auto &p : c->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
      if (p.first == 0) c->stats.sample_ms += ms;
      else if (p.first == 1) c->stats.grid_ms += ms;
      else c->stats.post_ms += ms;
    }
  }
  c->pending.clear();
  c->ev_next = 0;
}

#define CK(x)                                   \
  do {                                          \
    cudaError_t _e = (x);                       \
    if (_e != cudaSuccess) return SMC_ERR_CUDA; \
  } while (0)

smc_status validate(const smc_params &p) {
  if (p.which_mc_model != 5 && p.which_mc_model != 1 && p.which_mc_model != 7) return SMC_ERR_CONFIG;
  if (p.which_mc_model == 5 && p.sub_model != 1 && p.sub_model != 2) return SMC_ERR_CONFIG;
  if (p.shape_of_nucleons != 1 && p.shape_of_nucleons != 2 && p.shape_of_nucleons != 4) return SMC_ERR_CONFIG;
  if (p.shape_of_entropy != 1 && p.shape_of_entropy != 2) return SMC_ERR_CONFIG;
  if (p.collision_criterion != 1 && p.collision_criterion != 2) return SMC_ERR_CONFIG;
  if (p.Aproj < 1 || p.Atarg < 1 || p.Aproj > smc::kMaxA || p.Atarg > smc::kMaxA) return SMC_ERR_CONFIG;
  if (!(p.dx > 0) || !(p.dy > 0) || !(p.maxx > 0) || !(p.maxy > 0)) return SMC_ERR_CONFIG;
  if (p.ecc_from_order < 1 || p.ecc_to_order > 9 || p.ecc_from_order > p.ecc_to_order) return SMC_ERR_CONFIG;
  if (p.bmax < p.bmin || p.bmin < 0) return SMC_ERR_CONFIG;
  // multiplicity fluctuations: none, or the Gamma weights of model 6
  if (p.cc_fluctuation_model < 0 || (p.cc_fluctuation_model > 2 && p.cc_fluctuation_model != 6)) return SMC_ERR_CONFIG;
  if (p.cc_fluctuation_model == 6 && !(p.cc_fluctuation_gamma_theta > 0)) return SMC_ERR_CONFIG;
  if (p.cc_fluctuation_model == 1 && !(p.cc_fluctuation_k > 0)) return SMC_ERR_CONFIG;
  if (p.cc_fluctuation_model == 2 && p.which_mc_model == 7) return SMC_ERR_CONFIG;   // no T_A, T_B planes
  // inverse-CDF radii: spherical Woods-Saxon nuclei
  if (p.ws_inverse_cdf && (p.Aproj < 3 || p.Atarg < 3 || p.proj_deformed || p.targ_deformed)) return SMC_ERR_CONFIG;
  return SMC_OK;
}

// The quadrature of the MC-KLN tables (Gauss-Legendre nodes on [0,1] in
// p_T, k_T, phi; KLNModel's constants, src/KLNModel.cpp:27-90): the node
// arrays are copied to *d_nodes (device memory the caller frees).
smc_status kln_quadrature(Ctx *c, smc::KlnDev &K, double **d_nodes_out) {
  const smc_params &p = c->prm;
  int npt = p.kln_npt > 0 ? p.kln_npt : 48, nkt = p.kln_nkt > 0 ? p.kln_nkt : 64,
      nphi = p.kln_nphi > 0 ? p.kln_nphi : 32;
  std::vector<double> xp, wp, xk, wk, xf, wf;
  gauss_legendre01(npt, xp, wp);
  gauss_legendre01(nkt, xk, wk);
  gauss_legendre01(nphi, xf, wf);
  // cos(2 pi x) of the phi nodes up to the middle (the rule is symmetric)
  std::vector<double> cf(nphi / 2 + 1);
  for (int f = 0; f <= nphi / 2 && f < nphi; f++) cf[f] = std::cos(2 * M_PI * xf[f]);
  std::vector<double> nodes;
  for (auto *v : {&xp, &wp, &xk, &wk, &xf, &wf, &cf}) nodes.insert(nodes.end(), v->begin(), v->end());
  double *d_nodes = nullptr;
  CK(cudaMalloc(&d_nodes, sizeof(double) * nodes.size()));
  *d_nodes_out = d_nodes;
  CK(cudaMemcpyAsync(d_nodes, nodes.data(), sizeof(double) * nodes.size(), cudaMemcpyHostToDevice, c->st));
  K = smc::KlnDev{};
  K.ecm = p.ecm;
  K.lambda = p.lambda;
  K.y = 0.0;
  K.ptmin = 0.1;
  K.ptmax = 12.0;
  K.lambda_qcd2 = 0.2 * 0.2;
  K.alpha_max = 0.5;
  K.beta0 = (33.0 - 2.0 * 3.0) / (12 * M_PI);
  double CF = (3.0 * 3.0 - 1.0) / (2 * 3.0);
  K.fac = CF * 2. / (3. * M_PI * M_PI);
  const double hbarC = 0.197327053;
  K.prefactor = 1.0 * 2.0 * (2. / CF / (hbarC * hbarC)) * 9. / 32.;
  K.npt = npt; K.nkt = nkt; K.nphi = nphi;
  K.xp = d_nodes; K.wp = d_nodes + npt; K.xk = K.wp + npt; K.wk = K.xk + nkt; K.xf = K.wk + nkt;
  K.wf = K.xf + nphi;
  K.cf = K.wf + nphi;
  return SMC_OK;
}

smc_status build_kln_table(Ctx *c) {
  smc::KlnDev K;
  double *d_nodes = nullptr;
  smc_status s = kln_quadrature(c, K, &d_nodes);
  if (s) {
    if (d_nodes) cudaFree(d_nodes);
    return s;
  }
  int tmax = c->info.kln_tmax;
  CK(c->kln64.ensure((size_t)tmax * tmax));
  CK(c->kln32.ensure((size_t)tmax * tmax));
  CK(smc::launch_kln_table(K, tmax, c->info.kln_dT, c->kln64.p, c->kln32.p, c->st));
  CK(cudaStreamSynchronize(c->st));
  // the six-point polynomial of every table cell (sixPoint2dInterp,
  // src/arsenal.cpp:33-54) in FP64, rounded once: the per-cell lookup is
  // then two loads and five FMAs
  {
    std::vector<double> t((size_t)tmax * tmax);
    CK(cudaMemcpy(t.data(), c->kln64.p, sizeof(double) * t.size(), cudaMemcpyDeviceToHost));
    std::vector<float4> coef((size_t)tmax * tmax * 2, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int i = 0; i + 2 < tmax; i++)
      for (int j = 0; j + 2 < tmax; j++) {
        const double v00 = t[(size_t)i * tmax + j], v01 = t[(size_t)i * tmax + j + 1], v02 = t[(size_t)i * tmax + j + 2];
        const double v10 = t[(size_t)(i + 1) * tmax + j], v11 = t[(size_t)(i + 1) * tmax + j + 1];
        const double v20 = t[(size_t)(i + 2) * tmax + j];
        const double axx = 0.5 * (v00 - 2. * v10 + v20), axy = v00 - v01 - v10 + v11;
        const double ayy = 0.5 * (v00 - 2. * v01 + v02);
        const double bx = 0.5 * (-3. * v00 + 4. * v10 - v20), by = 0.5 * (-3. * v00 + 4. * v01 - v02);
        coef[2 * ((size_t)i * tmax + j)] = make_float4((float)axx, (float)axy, (float)ayy, (float)bx);
        coef[2 * ((size_t)i * tmax + j) + 1] = make_float4((float)by, (float)v00, 0.f, 0.f);
      }
    CK(c->kln_coef.ensure(coef.size()));
    CK(cudaMemcpy(c->kln_coef.p, coef.data(), sizeof(float4) * coef.size(), cudaMemcpyHostToDevice));
    c->P.kln_coef = c->kln_coef.p;
  }
  cudaFree(d_nodes);
  c->P.kln_table = c->kln32.p;
  return SMC_OK;
}

smc_status ensure_buffers(Ctx *c, int n, const smc_outputs *out) {
  const DevParams &P = c->P;
  CK(c->recs.ensure(n));
  CK(c->srcs.ensure((size_t)n * P.max_src));
  CK(c->status.ensure(n));
  if (!out->device) {
    size_t g = (size_t)P.nx * P.ny;
    if (out->ecc) CK(c->ecc.ensure((size_t)n * smc::kEccLen));
    if (out->rho) CK(c->rho.ensure((size_t)n * g));
    if (out->ta) CK(c->ta.ensure((size_t)n * g));
    if (out->tb) CK(c->tb.ensure((size_t)n * g));
    if (out->positions) CK(c->pos.ensure((size_t)n * 2 * (c->info.A + c->info.B)));
    if (out->wounded) CK(c->wounded.ensure((size_t)n * (c->info.A + c->info.B)));
    if (out->tangents) CK(c->ntan.ensure((size_t)n * 4 * (c->info.A + c->info.B)));
    if (out->collisions) CK(c->coll.ensure((size_t)n * 2 * P.max_coll));
    if (out->orientation) CK(c->orient.ensure((size_t)n * 4));
    if (out->rho_pt && c->pt_nbins > 0) CK(c->rho_pt.ensure((size_t)n * g * c->pt_nbins));
  }
  if (!out->ecc || out->device == 0) CK(c->ecc.ensure((size_t)n * smc::kEccLen));
  return SMC_OK;
}

// Gathers the small per-event scalars out of the event records.
__global__ void k_scalars(const EventRec *r, int n, int *npart, int *ncoll, double *b, int *attempts) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  if (npart) { npart[2 * e] = r[e].npart1; npart[2 * e + 1] = r[e].npart2; }
  if (ncoll) ncoll[e] = r[e].ncoll;
  if (b) b[e] = r[e].b;
  if (attempts) attempts[e] = r[e].attempts;
}

// The events of a chunk by decreasing source count (counting sort on
// nsrc / 8; the order within a bin does not matter: events are independent).
__global__ void k_order_events(const EventRec *recs, int n, int *order) {
  __shared__ int hist[1024];
  const int tid = threadIdx.x;
  for (int i = tid; i < 1024; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int e = tid; e < n; e += blockDim.x) atomicAdd(&hist[1023 - min(recs[e].nsrc >> 3, 1023)], 1);
  __syncthreads();
  if (tid == 0) {
    int acc = 0;
    for (int b = 0; b < 1024; b++) {
      const int c = hist[b];
      hist[b] = acc;
      acc += c;
    }
  }
  __syncthreads();
  for (int e = tid; e < n; e += blockDim.x) order[atomicAdd(&hist[1023 - min(recs[e].nsrc >> 3, 1023)], 1)] = e;
}

// Binary-collision positions of each event, in source order (the
// reference's order), one warp per event: out [n][max_coll][2].
__global__ void k_collisions(const EventRec *recs, const Source *srcs, int n, int max_src, int max_coll,
                             double *out) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int e = warp; e < n; e += nwarps) {
    const Source *S = srcs + (size_t)e * max_src;
    const int ns = recs[e].nsrc;
    double *o = out + (size_t)e * max_coll * 2;
    int pos = 0;
    for (int k0 = 0; k0 < ns; k0 += 32) {
      const int k = k0 + lane;
      const int kind = k < ns ? (S[k].kind & 15) : -1;
      const bool is = kind == smc::SRC_COLL || kind == smc::SRC_BINARY;
      const unsigned bal = __ballot_sync(0xffffffffu, is);
      if (is) {
        const int p = pos + __popc(bal & ((1u << lane) - 1u));
        if (p < max_coll) {
          o[2 * p] = S[k].x;
          o[2 * p + 1] = S[k].y;
        }
      }
      pos += __popc(bal);
    }
  }
}

// worst per-event status of a chunk into *worst (atomic max)
__global__ void k_status_max(const int *status, int n, int *worst) {
  int v = 0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) v = max(v, status[e]);
  for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v) atomicMax(worst, v);
}

// Batched splat of one chunk: the tensor-core contraction where the profile
// allows it, else the CUDA-core splat.
cudaError_t launch_splat(Ctx *c, const DevParams &P, int n, const EventRec *recs, const Source *srcs, float *rho,
                         float *ta, float *tb, float *scratch, double *ecc, int *status) {
  // the heaviest events first, each CTA taking the next event when it is free
  cudaError_t eo = c->ev_order.ensure(n);
  if (eo != cudaSuccess) return eo;
  k_order_events<<<1, 1024, 0, c->st>>>(recs, n, c->ev_order.p);
  eo = cudaGetLastError();
  if (eo != cudaSuccess) return eo;
  c->stats.launches++;
  if (c->use_tc && smc::grid_tc_supported(P)) {
    const size_t g = (size_t)P.nx * P.ny;
    cudaError_t e = c->corr_ev.ensure((size_t)c->sms * P.n_planes * g);
    if (e == cudaSuccess && !rho) e = c->rho_ev.ensure((size_t)n * g);
    if (e == cudaSuccess) e = c->cm_ev.ensure((size_t)n * 3);
    if (e != cudaSuccess) return e;
    c->stats.launches += P.no_moments ? 0 : 1;   // k_moments besides the timed launch
    return smc::launch_grid_tc(P, n, recs, srcs, rho, ta, tb, c->rho_ev.p, c->corr_ev.p, c->cm_ev.p, ecc, status,
                               c->sms, c->st, c->ev_order.p, c->tickets.p);
  }
  const int grid = std::max(1, std::min(n, c->sms * c->occ2));
  return smc::launch_grid(P, n, recs, srcs, rho, ta, tb, scratch, ecc, status, grid, c->st, c->ev_order.p,
                          c->tickets.p);
}

// One chunk of events through both stages.  Device outputs land directly in
// the caller's buffers at offset `off`; host outputs are staged and copied.
// per-event status codes written by the kernels -> API status
smc_status status_error(int worst) {
  switch (worst) {
    case 0: return SMC_OK;
    case 3: return SMC_ERR_RETRY_CAP;
    case 4: return SMC_ERR_KLN_TABLE;
    case 5: return SMC_ERR_ZERO_DNDY;
    case 6: return SMC_ERR_CAPACITY;
    default: return SMC_ERR_CUDA;
  }
}

smc_status run_chunk(Ctx *c, uint64_t first_event, int off, int n, const smc_outputs *out,
                     const double *inj_p, const double *inj_t, const double *inj_b, bool plain) {
  const DevParams &P = c->P;
  const size_t g = (size_t)P.nx * P.ny;
  const int AB = c->info.A + c->info.B;
  const bool dev = out->device != 0;
  double *ecc = dev && out->ecc ? out->ecc + (size_t)off * smc::kEccLen : c->ecc.p;
  float *rho = out->rho ? (dev ? out->rho + (size_t)off * g : c->rho.p) : nullptr;
  float *ta = out->ta ? (dev ? out->ta + (size_t)off * g : c->ta.p) : nullptr;
  float *tb = out->tb ? (dev ? out->tb + (size_t)off * g : c->tb.p) : nullptr;
  // p_T-differential densities: read the splat's thickness outputs
  const bool want_pt = out->rho_pt && c->pt_nbins > 0 && P.which_mc_model == 1;
  const size_t gpt = g * (size_t)c->pt_nbins;
  float *rho_pt = want_pt ? (dev ? out->rho_pt + (size_t)off * gpt : c->rho_pt.p) : nullptr;
  if (want_pt && !ta) {
    CK(c->pt_ta.ensure((size_t)n * g));
    ta = c->pt_ta.p;
  }
  if (want_pt && !tb) {
    CK(c->pt_tb.ensure((size_t)n * g));
    tb = c->pt_tb.p;
  }
  double *pos = out->positions ? (dev ? out->positions + (size_t)off * 2 * AB : c->pos.p) : nullptr;
  uint8_t *wnd = out->wounded ? (dev ? out->wounded + (size_t)off * AB : c->wounded.p) : nullptr;
  double *tg = out->tangents ? (dev ? out->tangents + (size_t)off * 4 * AB : c->ntan.p) : nullptr;
  double *ori = out->orientation ? (dev ? out->orientation + (size_t)off * 4 : c->orient.p) : nullptr;
  smc::TangentIO tio = c->tio;
  if (tg) tio.ntan = tg;
  tio.orient = ori;
  int grid1 = std::max(1, std::min(n, c->sms * c->occ1));
  int grid2 = std::max(1, std::min(n, c->sms * c->occ2));
  if (!rho) CK(c->scratch.ensure((size_t)(plain ? 1 : grid2) * g));
  if (plain) {
    for (int e = 0; e < n; e++) {
      smc::TangentIO te{};
      te.ntan = tg ? tg + (size_t)e * 4 * AB : nullptr;
      te.orient = ori ? ori + (size_t)e * 4 : nullptr;
      CK(timed(c, 0, [&] {
        return smc::launch_sample_pair_mixed(
            P, first_event + e, 1, inj_p ? inj_p + (size_t)e * 2 * c->info.A : nullptr,
            inj_t ? inj_t + (size_t)e * 2 * c->info.B : nullptr, inj_b ? inj_b + e : nullptr, c->recs.p + e,
            c->srcs.p + (size_t)e * P.max_src, pos ? pos + (size_t)e * 2 * AB : nullptr,
            wnd ? wnd + (size_t)e * AB : nullptr, nullptr, nullptr, nullptr, 1, c->st, &te);
      }));
      CK(timed(c, 1, [&] {
        return smc::launch_grid(P, 1, c->recs.p + e, c->srcs.p + (size_t)e * P.max_src,
                                rho ? rho + (size_t)e * g : nullptr, ta ? ta + (size_t)e * g : nullptr,
                                tb ? tb + (size_t)e * g : nullptr, c->scratch.p, ecc + (size_t)e * smc::kEccLen,
                                c->status.p + e, 1, c->st);
      }));
    }
  } else {
    CK(timed(c, 0, [&] {
      return smc::launch_sample_pair_mixed(P, first_event, n, inj_p, inj_t, inj_b, c->recs.p, c->srcs.p, pos, wnd,
                                           c->mix_sys.p && c->mixing ? c->mix_sys.p : nullptr,
                                           c->mixing ? c->mix_ev.p : nullptr, c->mixing ? c->mix_order.p : nullptr,
                                           grid1, c->st, &tio, nullptr, c->tickets.p + 2);
    }));
    CK(timed(c, 1, [&] {
      return launch_splat(c, P, n, c->recs.p, c->srcs.p, rho, ta, tb, c->scratch.p, ecc, c->status.p);
    }));
  }
  // per-event binary-collision and spectator densities: views of the
  // event's records splatted on their own (MCnucl::calculate_rho_binary,
  // calculate_spectator_density, src/MCnucl.cpp:481-614)
  const bool want_rhob = out->rho_binary != nullptr, want_spect = out->spectator_a || out->spectator_b;
  float *rhob = nullptr, *spa = nullptr, *spb = nullptr;
  if (want_rhob || want_spect) {
    CK(c->avg_view.ensure((size_t)n * P.max_src));
    CK(c->avg_vrecs.ensure(n));
    CK(c->avg_status.ensure(n));
    CK(c->scratch.ensure((size_t)c->sms * c->occ2 * g));
    if (!dev) CK(c->ev_aux.ensure((size_t)n * g * 3));
    rhob = want_rhob ? (dev ? out->rho_binary + (size_t)off * g : c->ev_aux.p) : nullptr;
    // both spectator planes are splatted; a plane not asked for lands in staging
    if (want_spect) {
      if (!dev || !out->spectator_a || !out->spectator_b) CK(c->ev_aux.ensure((size_t)n * g * 3));
      spa = dev && out->spectator_a ? out->spectator_a + (size_t)off * g : c->ev_aux.p + (size_t)n * g;
      spb = dev && out->spectator_b ? out->spectator_b + (size_t)off * g : c->ev_aux.p + (size_t)n * g * 2;
    }
    const int grid3 = std::max(1, std::min(n, c->sms * 4));
    if (want_rhob) {
      DevParams Pv = P;
      Pv.which_mc_model = 5;   // the plane is written out as it is
      Pv.nbd = 0;
      Pv.n_planes = 1;
      Pv.want_ta = Pv.want_tb = 0;
      Pv.no_moments = 1;
      CK(smc::launch_avg_view(Pv, n, c->recs.p, c->srcs.p, c->avg_view.p, 0, c->avg_vrecs.p, grid3, c->st));
      CK(timed(c, 2, [&] {
        return launch_splat(c, Pv, n, c->avg_vrecs.p, c->avg_view.p, rhob, nullptr, nullptr, c->scratch.p, c->ecc.p,
                            c->avg_status.p);   // (a view's own status is not the event's)
      }));
    }
    if (want_spect) {
      DevParams Pv = P;
      Pv.which_mc_model = 5;   // planes 1, 2 are written out as they are
      Pv.n_planes = 3;
      Pv.want_ta = Pv.want_tb = 1;
      Pv.no_moments = 1;
      Pv.nbd = 0;
      CK(smc::launch_avg_view(Pv, n, c->recs.p, c->srcs.p, c->avg_view.p, 1, c->avg_vrecs.p, grid3, c->st));
      CK(timed(c, 2, [&] {
        return launch_splat(c, Pv, n, c->avg_vrecs.p, c->avg_view.p, nullptr, spa, spb, c->scratch.p, c->ecc.p,
                            c->avg_status.p);
      }));
    }
  }
  if (want_pt) {
    CK(timed(c, 2, [&] {
      return smc::launch_kln_pt_cells(P, n, c->recs.p, c->srcs.p, ta, tb, c->pt32.p, c->pt_nbins, rho_pt,
                                      c->status.p, std::max(1, std::min(n, c->sms * 4)), c->st);
    }));
  }
  double *coll = out->collisions ? (dev ? out->collisions + (size_t)off * 2 * P.max_coll : c->coll.p) : nullptr;
  if (coll) {
    k_collisions<<<(n + 7) / 8, 256, 0, c->st>>>(c->recs.p, c->srcs.p, n, P.max_src, P.max_coll, coll);
    CK(cudaGetLastError());
    c->stats.launches++;
  }
  int *np = out->npart ? (dev ? out->npart + 2 * off : nullptr) : nullptr;
  int *nc = out->ncoll ? (dev ? out->ncoll + off : nullptr) : nullptr;
  double *bb = out->b ? (dev ? out->b + off : nullptr) : nullptr;
  int *at = out->attempts ? (dev ? out->attempts + off : nullptr) : nullptr;
  if (dev && (np || nc || bb || at)) {
    k_scalars<<<(n + 255) / 256, 256, 0, c->st>>>(c->recs.p, n, np, nc, bb, at);
    CK(cudaGetLastError());
    c->stats.launches++;
  }
  // status of every event of the chunk (also carries stage-1 failures)
  c->h_status.resize(n);
  CK(cudaMemcpyAsync(c->h_status.data(), c->status.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->st));
  if (!dev) {
    if (out->ecc)
      CK(cudaMemcpyAsync(out->ecc + (size_t)off * smc::kEccLen, ecc, sizeof(double) * n * smc::kEccLen,
                         cudaMemcpyDeviceToHost, c->st));
    if (out->rho) CK(cudaMemcpyAsync(out->rho + (size_t)off * g, rho, sizeof(float) * n * g, cudaMemcpyDeviceToHost, c->st));
    if (out->ta) CK(cudaMemcpyAsync(out->ta + (size_t)off * g, ta, sizeof(float) * n * g, cudaMemcpyDeviceToHost, c->st));
    if (out->tb) CK(cudaMemcpyAsync(out->tb + (size_t)off * g, tb, sizeof(float) * n * g, cudaMemcpyDeviceToHost, c->st));
    if (want_pt)
      CK(cudaMemcpyAsync(out->rho_pt + (size_t)off * gpt, rho_pt, sizeof(float) * n * gpt, cudaMemcpyDeviceToHost,
                         c->st));
    if (out->rho_binary)
      CK(cudaMemcpyAsync(out->rho_binary + (size_t)off * g, rhob, sizeof(float) * n * g, cudaMemcpyDeviceToHost,
                         c->st));
    if (out->spectator_a)
      CK(cudaMemcpyAsync(out->spectator_a + (size_t)off * g, spa, sizeof(float) * n * g, cudaMemcpyDeviceToHost,
                         c->st));
    if (out->spectator_b)
      CK(cudaMemcpyAsync(out->spectator_b + (size_t)off * g, spb, sizeof(float) * n * g, cudaMemcpyDeviceToHost,
                         c->st));
    if (out->positions)
      CK(cudaMemcpyAsync(out->positions + (size_t)off * 2 * AB, pos, sizeof(double) * n * 2 * AB,
                         cudaMemcpyDeviceToHost, c->st));
    if (out->wounded)
      CK(cudaMemcpyAsync(out->wounded + (size_t)off * AB, wnd, (size_t)n * AB, cudaMemcpyDeviceToHost, c->st));
    if (out->tangents)
      CK(cudaMemcpyAsync(out->tangents + (size_t)off * 4 * AB, tg, sizeof(double) * n * 4 * AB,
                         cudaMemcpyDeviceToHost, c->st));
    if (out->collisions)
      CK(cudaMemcpyAsync(out->collisions + (size_t)off * 2 * P.max_coll, coll, sizeof(double) * n * 2 * P.max_coll,
                         cudaMemcpyDeviceToHost, c->st));
    if (out->orientation)
      CK(cudaMemcpyAsync(out->orientation + (size_t)off * 4, ori, sizeof(double) * n * 4, cudaMemcpyDeviceToHost,
                         c->st));
    if (out->npart || out->ncoll || out->b || out->attempts) {
      c->h_recs.resize(n);
      CK(cudaMemcpyAsync(c->h_recs.data(), c->recs.p, sizeof(EventRec) * n, cudaMemcpyDeviceToHost, c->st));
    }
  }
  CK(cudaStreamSynchronize(c->st));
  collect_timing(c);
  c->stats.events += n;
  if (!dev) {
    for (int e = 0; e < n; e++) {
      const EventRec &r = c->h_recs.empty() ? EventRec{} : c->h_recs[std::min<size_t>(e, c->h_recs.size() - 1)];
      if (out->npart) { out->npart[2 * (off + e)] = r.npart1; out->npart[2 * (off + e) + 1] = r.npart2; }
      if (out->ncoll) out->ncoll[off + e] = r.ncoll;
      if (out->b) out->b[off + e] = r.b;
      if (out->attempts) out->attempts[off + e] = r.attempts;
    }
  }
  int worst = 0;
  for (int e = 0; e < n; e++) worst = std::max(worst, c->h_status[e]);
  return status_error(worst);
}

// Injected positions of events [off, off + m) staged on the device (NULLs
// when not injecting).
smc_status stage_injection(Ctx *c, int off, int m, const double *inj_p, const double *inj_t, const double *inj_b,
                           bool device, const double **ip, const double **it, const double **ib) {
  *ip = *it = *ib = nullptr;
  if (!inj_p) return SMC_OK;
  size_t np = (size_t)m * 2 * c->info.A, nt = (size_t)m * 2 * c->info.B;
  CK(c->inj_p.ensure(np));
  CK(c->inj_t.ensure(nt));
  cudaMemcpyKind kind = device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  CK(cudaMemcpyAsync(c->inj_p.p, inj_p + (size_t)off * 2 * c->info.A, sizeof(double) * np, kind, c->st));
  CK(cudaMemcpyAsync(c->inj_t.p, inj_t + (size_t)off * 2 * c->info.B, sizeof(double) * nt, kind, c->st));
  *ip = c->inj_p.p;
  *it = c->inj_t.p;
  if (inj_b) {
    CK(c->inj_b.ensure(m));
    CK(cudaMemcpyAsync(c->inj_b.p, inj_b + off, sizeof(double) * m, kind, c->st));
    *ib = c->inj_b.p;
  }
  return SMC_OK;
}

smc_status run(Ctx *c, uint64_t first_event, int n, const smc_outputs *out, const double *inj_p,
               const double *inj_t, const double *inj_b, bool plain) {
  if (n < 0 || !out) return SMC_ERR_ARGUMENT;
  if (n == 0) return SMC_OK;
  CK(cudaSetDevice(c->device));
  smc_status worst = SMC_OK;
  // p_T-differential densities take [nx][ny][bins] floats per event: their
  // chunks are kept to about 2^29 values
  int chunk = c->chunk;
  if (out->rho_pt && c->pt_nbins > 0) {
    const size_t per_ev = (size_t)c->P.nx * c->P.ny * c->pt_nbins;
    chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)chunk, ((size_t)1 << 29) / per_ev));
  }
  for (int off = 0; off < n; off += chunk) {
    int m = std::min(chunk, n - off);
    smc_status s = ensure_buffers(c, m, out);
    if (s) return s;
    const double *ip = nullptr, *it = nullptr, *ib = nullptr;
    s = stage_injection(c, off, m, inj_p, inj_t, inj_b, out->device != 0, &ip, &it, &ib);
    if (s) return s;
    s = run_chunk(c, first_event + off, off, m, out, ip, it, ib, plain);
    if (s && s != SMC_ERR_ZERO_DNDY) return s;
    if (s) worst = s;
  }
  return worst;
}

}  // namespace

extern "C" {

const char *smc_status_string(smc_status s) {
  switch (s) {
    case SMC_OK: return "ok";
    case SMC_ERR_ARGUMENT: return "invalid argument";
    case SMC_ERR_CONFIG: return "unsupported or inconsistent configuration";
    case SMC_ERR_RETRY_CAP: return "event retry cap reached";
    case SMC_ERR_KLN_TABLE: return "thickness beyond the KLN dN/dy table";
    case SMC_ERR_ZERO_DNDY: return "integrated density is zero";
    case SMC_ERR_CAPACITY: return "per-event collision capacity exceeded";
    case SMC_ERR_CUDA: return "CUDA runtime error";
    case SMC_ERR_NO_DEVICE: return "no usable GPU";
    case SMC_ERR_SCRATCH_LIMIT: return "request exceeds the fixed scratch of smc_inject_noalloc";
    default: return "unknown status";
  }
}

const char *smc_cuda_error_string(void) {
  thread_local char buf[256];
  const cudaError_t e = cudaGetLastError();
  std::snprintf(buf, sizeof buf, "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
  return buf;
}

smc_status smc_create(const smc_params *params, void **ctx_out) {
  if (!params || !ctx_out) return SMC_ERR_ARGUMENT;
  *ctx_out = nullptr;
  smc_status v = validate(*params);
  if (v) return v;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SMC_ERR_NO_DEVICE;
  Ctx *c = new (std::nothrow) Ctx;
  if (!c) return SMC_ERR_ARGUMENT;
  c->prm = *params;
  const smc_params &p = c->prm;
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
  if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) { delete c; return SMC_ERR_CUDA; }
  c->st = c->own;

  DevParams &P = c->P;
  const double sigin = derive_common(p, P);
  const double width = P.width;
  if (p.cc_fluctuation_model == 1 || p.cc_fluctuation_model == 2) {   // MCnucl.cpp:869-905
    const double hbarc = 0.197327053;
    P.nbd = p.cc_fluctuation_model;
    P.nbd_k = p.cc_fluctuation_k;
    P.nbd_kpp = 1.0 / M_PI * p.dx * p.dy * 1.0 * (0.25 * 0.25 / hbarc / hbarc);
  }
  if (p.ws_inverse_cdf) {
    for (int w = 0; w < 2; w++) {
      smc::NucleusDev &n = P.nuc[w];
      std::vector<double> tab;
      icdf_table(n, tab);
      if (c->icdf_tab[w].ensure(tab.size()) != cudaSuccess ||
          cudaMemcpy(c->icdf_tab[w].p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice) !=
              cudaSuccess) {
        smc_destroy(c);
        return SMC_ERR_CUDA;
      }
      n.icdf = c->icdf_tab[w].p;
    }
  }
  P.max_attempts = p.max_attempts > 0 ? p.max_attempts : 100000;
  P.max_coll = p.max_collisions > 0 ? p.max_collisions : 4096;
  P.max_src = 2 * (p.Aproj + p.Atarg) + P.max_coll;
  P.want_ta = P.want_tb = 0;
  P.n_planes = p.which_mc_model == 5 ? 1 : 2;   // smallest layout, checked below; T_A/T_B requests at each call
  const double d_max = p.shape_of_nucleons == 1 ? 2. * std::sqrt(P.dsq) : 5. * width;
  if (p.which_mc_model == 1) {
    int sub = p.tmax_subdivision > 0 ? p.tmax_subdivision : 3;
    int tmax = p.tmax > 1 ? p.tmax : 71;
    P.kln_tmax = (p.shape_of_nucleons >= 2) ? sub * (tmax - 1) + 1 : tmax;   // MCnucl.cpp:915-919
    P.kln_dT = 10.0 / sigin / 1 / ((p.shape_of_nucleons >= 2) ? sub : 1);
    P.kln_dT_f = (float)P.kln_dT;
    P.kln_inv_dT_f = (float)(1.0 / P.kln_dT);
    // Relative error bound of a Gaussian term of the splats' FP32 thickness
    // against the FP64 one.  A source sits at grid cell + fraction (FP64
    // split, the fraction rounded by 2^-25 grid units), and the grid
    // distance d = (k - cell) - fraction errs by 2^-25 + 2^-24 |d|; the
    // exponent d^2 c (c = spacing^2 log2(e) / 2w^2 rounded, two products)
    // then errs by 2^-24 (c |d| + 5 d^2 c) per axis, at most 2^-24 (c
    // 5w/spacing + 5 x 12.5 log2(e)) in all (r <= 5w), times ln 2 relative;
    // ex2.approx adds 2^-22 per factor, the weight and the two products an
    // ulp each, the tensor cores' split-TF32 products below 1e-6.  Plus the
    // quotient by dT (T times the rounded 1/dT: 2 ulp) and a margin.  The
    // kernels add one rounding per summed term, at most max(Npart1, Npart2)
    // terms per event.  Disk nucleons add one constant per term.
    const double u = std::ldexp(1.0, -24), ln2 = std::log(2.0);
    const double cg = std::max(p.dx, p.dy) * std::max(p.dx, p.dy) / (2 * width * width) / ln2;
    const double expo = u * (cg * 5 * width / std::min(p.dx, p.dy) + 5 * 12.5 / ln2) * ln2;
    const double terms = p.shape_of_nucleons == 1 ? 1e-7 : expo + 2 * std::ldexp(1.0, -22) + 3 * u + 1e-6;
    P.kln_band = (float)(terms + 1e-6);
    if (p.kln_exact_band > P.kln_band) P.kln_band = (float)p.kln_exact_band;
    P.kln_tzero = (float)(0.5 * (p.shape_of_nucleons == 1 ? 10.0 / sigin : P.peak * std::exp(-12.5)));
  }
  smc_info &I = c->info;
  I.nx = P.nx; I.ny = P.ny; I.sigin = sigin; I.dsq = P.dsq; I.width = width; I.sigma_gg = P.sigma_gg;
  I.kln_tmax = P.kln_tmax; I.kln_dT = P.kln_dT; I.A = p.Aproj; I.B = p.Atarg; I.max_collisions = P.max_coll;

  if (c->tickets.ensure(4) != cudaSuccess) { smc_destroy(c); return SMC_ERR_CUDA; }
  size_t smem2 = smc::grid_smem(P);
  cudaDeviceGetAttribute(&c->dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  if ((int)smem2 > c->dev_smem) { smc_destroy(c); return SMC_ERR_CONFIG; }
  // persistent grid sizes from the occupancy the kernels reach
  c->occ1 = std::max(1, (int)(227 * 1024 / (smc::sample_pair_smem() + 1024)));
  c->occ1 = std::min(c->occ1, 8);
  c->occ2 = 1;
  if (p.which_mc_model == 1) {
    smc_status s = build_kln_table(c);
    if (s) { smc_destroy(c); return s; }
  }
  *ctx_out = c;
  return SMC_OK;
}

void smc_destroy(void *ctx) {
  Ctx *c = static_cast<Ctx *>(ctx);
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  c->recs.release(); c->srcs.release(); c->ecc.release(); c->pos.release(); c->bvec.release(); c->coll.release();
  c->inj_p.release(); c->inj_t.release(); c->inj_b.release(); c->rho.release(); c->ta.release();
  c->tb.release(); c->scratch.release(); c->status.release(); c->npart.release(); c->ncoll.release();
  c->attempts.release(); c->wounded.release(); c->rho_ev.release(); c->corr_ev.release(); c->cm_ev.release();
  c->mix_sys.release(); c->mix_ev.release(); c->mix_order.release(); c->kln64.release(); c->kln32.release();
  c->kln_coef.release();
  c->pt64.release(); c->pt32.release(); c->pt_ta.release(); c->pt_tb.release(); c->rho_pt.release();
  c->ev_aux.release();
  c->avg_state.release(); c->avg_rho.release(); c->avg_acc.release();
  c->avg_ta.release(); c->avg_tb.release(); c->avg_aux.release(); c->avg_view.release(); c->avg_vrecs.release(); c->avg_status.release();
  c->avg_frame.release(); c->avg_order.release(); c->avg_seg.release(); c->avg_count.release();
  c->avg_edges.release(); c->avg_bins.release(); c->avg_part.release();
  c->ev_order.release(); c->tickets.release();
  c->adj_rho.release(); c->adj_lam.release(); c->adj_grho.release(); c->adj_geps.release(); c->adj_out.release();
  c->icdf_tab[0].release(); c->icdf_tab[1].release(); c->ntan.release(); c->inj_tp.release(); c->inj_tt.release();
  c->stan.release();
  for (auto &t : c->conf) t.second.xyz.release();
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->mgraph) cudaGraphExecDestroy(c->mgraph);
  c->mg_sys.release(); c->mg_ev.release(); c->mg_order.release();
  c->ev_base.release(); c->worst.release();
  if (c->h_first) cudaFreeHost(c->h_first);
  if (c->h_worst) cudaFreeHost(c->h_worst);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
}

smc_status smc_get_info(void *ctx, smc_info *info) {
  if (!ctx || !info) return SMC_ERR_ARGUMENT;
  *info = static_cast<Ctx *>(ctx)->info;
  return SMC_OK;
}

smc_status smc_set_stream(void *ctx, void *cuda_stream) {
  if (!ctx) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  c->st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->own;
  return SMC_OK;
}

smc_status smc_synchronize(void *ctx) {
  if (!ctx) return SMC_ERR_ARGUMENT;
  return cudaStreamSynchronize(static_cast<Ctx *>(ctx)->st) == cudaSuccess ? SMC_OK : SMC_ERR_CUDA;
}

static smc_status set_thickness_flags(Ctx *c, const smc_outputs *out) {
  DevParams &P = c->P;
  // model-2 NBD fluctuations of the Glauber density need T_A, T_B per cell
  const bool nbd_thick = P.nbd == 2 && P.which_mc_model == 5;
  P.want_ta = out->ta != nullptr || nbd_thick;
  P.want_tb = out->tb != nullptr || nbd_thick;
  // collision records whatever the model (collision positions, rho_binary)
  P.want_binary = out->collisions != nullptr || out->rho_binary != nullptr;
  P.want_spect = out->spectator_a != nullptr || out->spectator_b != nullptr;   // spectator records
  if ((out->ta || out->tb) && P.which_mc_model == 7) return SMC_ERR_CONFIG;
  // splat planes: Glauber rho (+ T_A, T_B on request); MC-KLN T_A, T_B;
  // sqrt(T_A T_B) scaling rho_A, rho_B
  P.n_planes = P.which_mc_model == 5 ? ((P.want_ta || P.want_tb) ? 3 : 1) : 2;
  if (P.ny > 512) return SMC_ERR_CONFIG;
  // the CUDA-core splat's accumulator strip must fit (T_A, T_B on a wide grid may not)
  if ((int)smc::grid_smem(P) > c->dev_smem) return SMC_ERR_CONFIG;
  c->occ2 = smc::grid_blocks_per_sm(P);
  return SMC_OK;
}


smc_status smc_generate(void *ctx, uint64_t first_event, int n, const smc_outputs *out) {
  if (!ctx || !out) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  smc_status s = set_thickness_flags(c, out);
  if (s) return s;
  return run(c, first_event, n, out, nullptr, nullptr, nullptr, false);
}

smc_status smc_generate_plain(void *ctx, uint64_t first_event, int n, const smc_outputs *out) {
  if (!ctx || !out) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  smc_status s = set_thickness_flags(c, out);
  if (s) return s;
  return run(c, first_event, n, out, nullptr, nullptr, nullptr, true);
}

// A nucleus takes its mass number's configuration table, if the context has one.
void attach_configurations(const Ctx *c, smc::NucleusDev &n) {
  auto it = c->conf.find(n.A);
  const bool on = n.A >= 3 && it != c->conf.end() && it->second.n > 0;
  n.conf = on ? it->second.xyz.p : nullptr;
  n.nconf = on ? it->second.n : 0;
}

// The per-system table of a mixed batch (and each system's cost, A + B, and
// the largest A + B), after checking that the systems differ from the
// context's parameters only where a mixed batch allows it.
smc_status mixed_systems(Ctx *c, const smc_params *systems, int nsys, int n, const int *system_of_event,
                         const smc_outputs *out, std::vector<smc::SystemDev> &sys, std::vector<int> &cost,
                         int &max_ab) {
  if (c->prm.ws_inverse_cdf) return SMC_ERR_CONFIG;
  if (out->tangents) return SMC_ERR_ARGUMENT;
  if (!systems || nsys < 1 || nsys > 64 || n < 0 || (n > 0 && !system_of_event)) return SMC_ERR_ARGUMENT;
  if (out->positions || out->wounded) return SMC_ERR_ARGUMENT;   // per-system shapes
  const smc_params &q = c->prm;
  if (q.which_mc_model == 1 || q.shape_of_nucleons != 4) return SMC_ERR_CONFIG;
  sys.assign(nsys, smc::SystemDev{});
  cost.assign(nsys, 0);
  max_ab = c->info.A + c->info.B;
  for (int k = 0; k < nsys; k++) {
    const smc_params &p = systems[k];
    smc_status v = validate(p);
    if (v) return v;
    // everything but the nuclei, the energy / sigma_in, the impact-parameter
    // range and the Npart cut is the context's
    if (p.which_mc_model != q.which_mc_model || p.sub_model != q.sub_model ||
        p.shape_of_nucleons != q.shape_of_nucleons || p.shape_of_entropy != q.shape_of_entropy ||
        p.collision_criterion != q.collision_criterion || p.gauss_nucl_width != q.gauss_nucl_width ||
        p.quark_width != q.quark_width || p.alpha != q.alpha || p.maxx != q.maxx || p.maxy != q.maxy ||
        p.dx != q.dx || p.dy != q.dy || p.final_factor != q.final_factor ||
        p.ecc_from_order != q.ecc_from_order || p.ecc_to_order != q.ecc_to_order || p.seed != q.seed)
      return SMC_ERR_CONFIG;
    smc::SystemDev &d = sys[k];
    const double sigin = p.sigin_override > 0 ? p.sigin_override : sigma_inelastic(p.ecm);
    d.nuc[0] = make_nucleus(p.Aproj, p.proj_deformed, p.proj_R, p.proj_a, p.proj_d_min);
    d.nuc[1] = make_nucleus(p.Atarg, p.targ_deformed, p.targ_R, p.targ_a, p.targ_d_min);
    attach_configurations(c, d.nuc[0]);
    attach_configurations(c, d.nuc[1]);
    d.dsq = 0.1 * sigin / M_PI;   // MCnucl.cpp:120
    d.sigin = sigin;
    d.sigma_gg = sigma_gg_from(sigin, c->P.width);
    d.bmin = p.bmin; d.bmax = p.bmax; d.npmin = p.npmin; d.npmax = p.npmax;
    cost[k] = p.Aproj + p.Atarg;
    max_ab = std::max(max_ab, p.Aproj + p.Atarg);
  }
  for (int e = 0; e < n; e++)
    if (system_of_event[e] < 0 || system_of_event[e] >= nsys) return SMC_ERR_ARGUMENT;
  return SMC_OK;
}

// The order in which the CTAs take the events of chunk [off, off + m): heavy
// systems first.
void mixed_order(const std::vector<int> &cost, const int *system_of_event, int off, int m, std::vector<int> &order) {
  order.resize(m);
  for (int e = 0; e < m; e++) order[e] = e;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return cost[system_of_event[off + a]] > cost[system_of_event[off + b]];
  });
}

smc_status smc_generate_mixed(void *ctx, const smc_params *systems, int nsys, uint64_t first_event, int n,
                              const int *system_of_event, const smc_outputs *out) {
  if (!ctx || !out) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  std::vector<smc::SystemDev> sys;
  std::vector<int> cost;
  int max_ab = 0;
  smc_status s = mixed_systems(c, systems, nsys, n, system_of_event, out, sys, cost, max_ab);
  if (s) return s;
  s = set_thickness_flags(c, out);
  if (s) return s;
  if (n == 0) return SMC_OK;
  CK(cudaSetDevice(c->device));
  CK(c->mix_sys.ensure(nsys));
  CK(cudaMemcpyAsync(c->mix_sys.p, sys.data(), sizeof(smc::SystemDev) * nsys, cudaMemcpyHostToDevice, c->st));
  // per-event source capacity of the largest system
  const int saved_max_src = c->P.max_src;
  c->P.max_src = 2 * max_ab + c->P.max_coll;
  c->mixing = true;
  smc_status worst = SMC_OK;
  std::vector<int> order, evs;
  for (int off = 0; off < n; off += c->chunk) {
    const int m = std::min(c->chunk, n - off);
    mixed_order(cost, system_of_event, off, m, order);   // heavy systems first
    s = ensure_buffers(c, m, out);
    if (!s && (c->mix_ev.ensure(m) != cudaSuccess || c->mix_order.ensure(m) != cudaSuccess)) s = SMC_ERR_CUDA;
    if (!s && (cudaMemcpyAsync(c->mix_ev.p, system_of_event + off, sizeof(int) * m, cudaMemcpyHostToDevice, c->st) !=
                   cudaSuccess ||
               cudaMemcpyAsync(c->mix_order.p, order.data(), sizeof(int) * m, cudaMemcpyHostToDevice, c->st) !=
                   cudaSuccess))
      s = SMC_ERR_CUDA;
    if (!s) s = run_chunk(c, first_event + off, off, m, out, nullptr, nullptr, nullptr, false);
    if (s) worst = s;
    if (s && s != SMC_ERR_ZERO_DNDY) break;
  }
  c->mixing = false;
  c->P.max_src = saved_max_src;
  return worst;
}

smc_status smc_inject(void *ctx, int n, const double *xy_proj, const double *xy_targ, const double *b,
                      const smc_outputs *out) {
  if (!ctx || !out || !xy_proj || !xy_targ) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  smc_status s = set_thickness_flags(c, out);
  if (s) return s;
  return run(c, 0, n, out, xy_proj, xy_targ, b, false);
}

smc_status smc_adjoint(void *ctx, uint64_t first_event, int n, const double *xy_proj, const double *xy_targ,
                       const double *b, const smc_adjoint_args *ct, double *grad) {
  if (!ctx || !ct || !grad || n < 0 || (xy_proj && !xy_targ)) return SMC_ERR_ARGUMENT;
  if (!xy_proj && ct->tangent_proj) return SMC_ERR_ARGUMENT;
  if ((ct->tangent_proj != nullptr) != (ct->tangent_targ != nullptr)) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  for (int k = 0; k < 4; k++) grad[k] = 0.0;
  const smc_params &p = c->prm;
  if (p.which_mc_model != 5 || p.shape_of_entropy == 1 || (p.sub_model != 1 && p.sub_model != 2))
    return SMC_ERR_CONFIG;
  if (n == 0) return SMC_OK;
  CK(cudaSetDevice(c->device));
  smc_outputs none{};
  smc_status s = set_thickness_flags(c, &none);
  if (s) return s;
  const DevParams &P = c->P;
  const size_t g = (size_t)P.nx * P.ny;
  const bool dev = ct->device != 0;
  const int nb = smc::adjoint_blocks_per_sm(P);
  const int A = c->info.A, B = c->info.B;
  // positions depend on (R, a): inverse-CDF sampling, or injected tangents
  const bool tangents = xy_proj ? ct->tangent_proj != nullptr : c->prm.ws_inverse_cdf != 0;
  smc_status worst = SMC_OK;
  for (int off = 0; off < n; off += c->chunk) {
    const int m = std::min(c->chunk, n - off);
    const int grid = std::max(1, std::min(m, c->sms * nb));
    CK(c->adj_rho.ensure((size_t)m * g));
    CK(c->adj_lam.ensure((size_t)grid * g));
    CK(c->adj_out.ensure((size_t)m * 4));
    smc_outputs o{};
    o.device = 1;
    o.rho = c->adj_rho.p;
    s = ensure_buffers(c, m, &o);
    if (s) return s;
    const double *ip, *it, *ib;
    s = stage_injection(c, off, m, xy_proj, xy_targ, b, dev, &ip, &it, &ib);
    if (s) return s;
    smc::TangentIO tio{};
    if (tangents) {
      CK(c->ntan.ensure((size_t)m * 4 * (A + B)));
      CK(c->stan.ensure((size_t)m * P.max_src));
      tio.ntan = c->ntan.p;
      tio.stan = c->stan.p;
      if (xy_proj) {
        const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        CK(c->inj_tp.ensure((size_t)m * 4 * A));
        CK(c->inj_tt.ensure((size_t)m * 4 * B));
        CK(cudaMemcpyAsync(c->inj_tp.p, ct->tangent_proj + (size_t)off * 4 * A, sizeof(double) * m * 4 * A, kind,
                           c->st));
        CK(cudaMemcpyAsync(c->inj_tt.p, ct->tangent_targ + (size_t)off * 4 * B, sizeof(double) * m * 4 * B, kind,
                           c->st));
        tio.inj_proj = c->inj_tp.p;
        tio.inj_targ = c->inj_tt.p;
      }
    }
    // forward pass of the chunk (the densities are recomputed, not kept
    // between the forward call and this one)
    c->tio = tio;
    s = run_chunk(c, first_event + off, 0, m, &o, ip, it, ib, false);
    c->tio = smc::TangentIO{};
    if (s && s != SMC_ERR_ZERO_DNDY) return s;
    if (s) worst = s;
    const double *geps = nullptr;
    const float *grho = nullptr;
    if (ct->g_eps) {
      if (dev) {
        geps = ct->g_eps + (size_t)off * 2;
      } else {
        CK(c->adj_geps.ensure((size_t)m * 2));
        CK(cudaMemcpyAsync(c->adj_geps.p, ct->g_eps + (size_t)off * 2, sizeof(double) * m * 2,
                           cudaMemcpyHostToDevice, c->st));
        geps = c->adj_geps.p;
      }
    }
    if (ct->g_rho) {
      if (dev) {
        grho = ct->g_rho + (size_t)off * g;
      } else {
        CK(c->adj_grho.ensure((size_t)m * g));
        CK(cudaMemcpyAsync(c->adj_grho.p, ct->g_rho + (size_t)off * g, sizeof(float) * m * g,
                           cudaMemcpyHostToDevice, c->st));
        grho = c->adj_grho.p;
      }
    }
    CK(timed(c, 2, [&] {
      // the splat's heaviest-first order of the chunk, one ticket per event
      return smc::launch_adjoint(P, m, c->recs.p, c->srcs.p, tangents ? c->stan.p : nullptr, c->adj_rho.p, grho,
                                 geps, c->adj_lam.p, c->adj_out.p, grid, c->st, c->ev_order.p, c->tickets.p + 3);
    }));
    c->h_adj.resize((size_t)m * 4);
    CK(cudaMemcpyAsync(c->h_adj.data(), c->adj_out.p, sizeof(double) * m * 4, cudaMemcpyDeviceToHost, c->st));
    if (ct->grad_events)
      CK(cudaMemcpyAsync(ct->grad_events + (size_t)off * 4, c->adj_out.p, sizeof(double) * m * 4,
                         dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    collect_timing(c);
    for (int e = 0; e < m; e++)
      for (int k = 0; k < 4; k++) grad[k] += c->h_adj[(size_t)e * 4 + k];
  }
  return worst;
}

smc_status smc_average_profiles(void *ctx, uint64_t first_event, int n, const double *xy_proj,
                                const double *xy_targ, const double *b, int from_order, int to_order,
                                const smc_average_outputs *o, int *n_used) {
  if (!ctx || !o || n < 0 || from_order < 1 || to_order < from_order || (xy_proj && !xy_targ))
    return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  if (n_used) *n_used = 0;
  if (n == 0) return SMC_OK;
  CK(cudaSetDevice(c->device));
  // what to produce: [kind][frame] host grids, frame 0 = participant plane, 1 = reaction plane
  enum { K_SD, K_TA, K_TB, K_TATB, K_RHOB, K_SPA, K_SPB, K_N };
  double *const want[K_N][2] = {{o->sd, o->sd_rp},           {o->ta, o->ta_rp},
                                {o->tb, o->tb_rp},           {o->ta_tb, o->ta_tb_rp},
                                {o->rho_binary, o->rho_binary_rp}, {o->spectator_a, o->spectator_a_rp},
                                {o->spectator_b, o->spectator_b_rp}};
  bool frame_on[2] = {false, false}, kind_on[K_N] = {};
  for (int k = 0; k < K_N; k++)
    for (int f = 0; f < 2; f++)
      if (want[k][f]) { frame_on[f] = true; kind_on[k] = true; }
  if (!frame_on[0] && !frame_on[1]) return SMC_ERR_ARGUMENT;
  const bool thick = kind_on[K_TA] || kind_on[K_TB] || kind_on[K_TATB];
  if (thick && c->P.which_mc_model == 7) return SMC_ERR_CONFIG;
  // T_A, T_B from the thickness records splatted beside the density
  smc_outputs req{};
  float dummy = 0.f;
  if (thick) req.ta = req.tb = &dummy;
  smc_status s = set_thickness_flags(c, &req);
  if (s) return s;
  DevParams P = c->P;
  P.no_moments = 1;
  P.want_spect = kind_on[K_SPA] || kind_on[K_SPB];
  P.want_binary = kind_on[K_RHOB];
  const size_t g = (size_t)P.nx * P.ny;
  const int norders = to_order - from_order + 1;
  const size_t slab = g * norders;   // one kind and frame
  CK(c->avg_acc.ensure(slab * K_N * 2));
  CK(cudaMemsetAsync(c->avg_acc.p, 0, sizeof(double) * slab * K_N * 2, c->st));
  auto acc_of = [&](int k, int f, int q) { return c->avg_acc.p + ((size_t)(k * 2 + f) * norders + q) * g; };
  int used = 0;
  for (int off = 0; off < n; off += c->chunk) {
    const int m = std::min(c->chunk, n - off);
    CK(c->recs.ensure(m));
    CK(c->srcs.ensure((size_t)m * P.max_src));
    CK(c->status.ensure(m));
    CK(c->avg_state.ensure((size_t)m * P.max_src));
    CK(c->avg_rho.ensure((size_t)m * g));
    CK(c->ecc.ensure((size_t)m * smc::kEccLen));
    if (thick) { CK(c->avg_ta.ensure((size_t)m * g)); CK(c->avg_tb.ensure((size_t)m * g)); }
    if (P.want_spect || P.want_binary) {
      CK(c->avg_view.ensure((size_t)m * P.max_src));
      CK(c->avg_vrecs.ensure(m));
      CK(c->avg_status.ensure(m));
      CK(c->avg_aux.ensure((size_t)m * g * 2));
      CK(c->scratch.ensure((size_t)c->sms * c->occ2 * g));
    }
    const double *ip, *it, *ib;
    s = stage_injection(c, off, m, xy_proj, xy_targ, b, false, &ip, &it, &ib);
    if (s) return s;
    const int grid1 = std::max(1, std::min(m, c->sms * c->occ1));
    const int grid3 = std::max(1, std::min(m, c->sms * 4));
    auto splat = [&]() {
      return timed(c, 1, [&] {
        return launch_splat(c, P, m, c->recs.p, c->srcs.p, c->avg_rho.p, thick ? c->avg_ta.p : nullptr,
                            thick ? c->avg_tb.p : nullptr, nullptr, c->ecc.p, c->status.p);
      });
    };
    // the grids of one frame after its transform and splat
    auto accumulate = [&](int f, int q) -> smc_status {
      if (want[K_SD][f]) CK(smc::launch_avg_accum(c->avg_rho.p, m, g, acc_of(K_SD, f, q), c->st));
      if (want[K_TA][f]) CK(smc::launch_avg_accum(c->avg_ta.p, m, g, acc_of(K_TA, f, q), c->st));
      if (want[K_TB][f]) CK(smc::launch_avg_accum(c->avg_tb.p, m, g, acc_of(K_TB, f, q), c->st));
      if (want[K_TATB][f])
        CK(smc::launch_avg_accum_prod(c->avg_ta.p, c->avg_tb.p, m, g, acc_of(K_TATB, f, q), c->st));
      if (want[K_RHOB][f]) {   // MCnucl::calculate_rho_binary on the moved collisions
        DevParams Pv = P;
        Pv.which_mc_model = 5;   // the plane is written out as it is
        Pv.n_planes = 1;
        Pv.want_ta = Pv.want_tb = 0;
        Pv.nbd = 0;
        CK(smc::launch_avg_view(Pv, m, c->recs.p, c->srcs.p, c->avg_view.p, 0, c->avg_vrecs.p, grid3, c->st));
        CK(launch_splat(c, Pv, m, c->avg_vrecs.p, c->avg_view.p, c->avg_aux.p, nullptr, nullptr, c->scratch.p, c->ecc.p,
                        c->avg_status.p));   // (a view's own status, e.g. zero density, is not the event's)
        CK(smc::launch_avg_accum(c->avg_aux.p, m, g, acc_of(K_RHOB, f, q), c->st));
      }
      if (want[K_SPA][f] || want[K_SPB][f]) {   // MCnucl::calculate_spectator_density
        DevParams Pv = P;
        Pv.which_mc_model = 5;   // planes 1, 2 are written out as they are
        Pv.n_planes = 3;
        Pv.want_ta = Pv.want_tb = 1;
        Pv.nbd = 0;
        CK(smc::launch_avg_view(Pv, m, c->recs.p, c->srcs.p, c->avg_view.p, 1, c->avg_vrecs.p, grid3, c->st));
        CK(launch_splat(c, Pv, m, c->avg_vrecs.p, c->avg_view.p, nullptr, c->avg_aux.p, c->avg_aux.p + (size_t)m * g,
                        c->scratch.p, c->ecc.p, c->avg_status.p));
        if (want[K_SPA][f]) CK(smc::launch_avg_accum(c->avg_aux.p, m, g, acc_of(K_SPA, f, q), c->st));
        if (want[K_SPB][f])
          CK(smc::launch_avg_accum(c->avg_aux.p + (size_t)m * g, m, g, acc_of(K_SPB, f, q), c->st));
      }
      return SMC_OK;
    };
    CK(timed(c, 0, [&] {
      return smc::launch_sample_pair(P, xy_proj ? 0 : first_event + off, m, ip, it, ib, c->recs.p, c->srcs.p,
                                     nullptr, nullptr, grid1, c->st);
    }));
    CK(smc::launch_avg_init(P, m, c->recs.p, c->srcs.p, c->avg_state.p, grid3, c->st));
    CK(splat());   // MakeDensity.cpp:1275
    for (int q = 0; q < norders; q++) {
      const int order = from_order + q;
      if (frame_on[1]) {    // MakeDensity.cpp:1289-1330
        CK(smc::launch_avg_transform(P, m, c->recs.p, c->srcs.p, c->avg_state.p, c->avg_rho.p, order, 0, grid3,
                                     c->st));
        CK(splat());
        s = accumulate(1, q);
        if (s) return s;
      }
      // MakeDensity.cpp:1331-1386
      CK(smc::launch_avg_transform(P, m, c->recs.p, c->srcs.p, c->avg_state.p, c->avg_rho.p, order, 1, grid3,
                                   c->st));
      CK(splat());
      if (frame_on[0]) {
        s = accumulate(0, q);
        if (s) return s;
      }
    }
    c->stats.launches += 1;
    c->h_status.resize(m);
    c->h_recs.resize(m);
    CK(cudaMemcpyAsync(c->h_status.data(), c->status.p, sizeof(int) * m, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(c->h_recs.data(), c->recs.p, sizeof(EventRec) * m, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    collect_timing(c);
    c->stats.events += m;
    int worst = 0;
    for (int e = 0; e < m; e++) {
      // only events with a collision enter the mean; an injected event
      // without one has an empty density, which is not an error here
      const bool hit = c->h_recs[e].ncoll > 0;
      used += hit;
      worst = std::max(worst, (!hit && c->h_status[e] == 5) ? 0 : c->h_status[e]);
    }
    if (worst) return status_error(worst);
  }
  if (n_used) *n_used = used;
  std::vector<double> h(slab * K_N * 2);
  CK(cudaMemcpyAsync(h.data(), c->avg_acc.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  // means over the events with a collision; the entropy density is
  // getRho * finalFactor (MakeDensity::setSd, src/MakeDensity.cpp:2514-2522)
  for (int k = 0; k < K_N; k++)
    for (int f = 0; f < 2; f++) {
      if (!want[k][f]) continue;
      const double scale = used ? (k == K_SD ? c->P.final_factor : 1.0) / used : 0.0;
      const double *src = h.data() + (size_t)(k * 2 + f) * slab;
      for (size_t i = 0; i < slab; i++) want[k][f][i] = src[i] * scale;
    }
  return SMC_OK;
}

smc_status smc_average(void *ctx, uint64_t first_event, int n, const double *xy_proj, const double *xy_targ,
                       const double *b, int from_order, int to_order, int reaction_plane, double *mean,
                       double *mean_rp, int *n_used) {
  if (!mean) return SMC_ERR_ARGUMENT;
  smc_average_outputs o{};
  o.sd = mean;
  o.sd_rp = reaction_plane ? mean_rp : nullptr;
  return smc_average_profiles(ctx, first_event, n, xy_proj, xy_targ, b, from_order, to_order, &o, n_used);
}

smc_status smc_average_binned(void *ctx, uint64_t first_event, int n, int order, int method, int nbins,
                              const int *npart_edges, double *mean, int *counts) {
  if (!ctx || !mean || !npart_edges || n < 0 || order < 1 || order > 9 || nbins < 1 || nbins > 64 ||
      (method != 0 && method != 1))
    return SMC_ERR_ARGUMENT;
  for (int k = 0; k < nbins; k++)
    if (npart_edges[k] > npart_edges[k + 1]) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  CK(cudaSetDevice(c->device));
  smc_outputs none{};
  smc_status s = set_thickness_flags(c, &none);
  if (s) return s;
  DevParams P = c->P;
  P.no_moments = 1;
  const size_t g = (size_t)P.nx * P.ny;
  CK(c->avg_bins.ensure(g * nbins));
  const int slices = smc::avg_binned_slices(P);
  if (slices > 1) CK(c->avg_part.ensure(g * nbins * slices));
  CK(c->avg_count.ensure(nbins));
  CK(c->avg_seg.ensure(nbins + 1));
  CK(c->avg_edges.ensure(nbins + 1));
  CK(cudaMemsetAsync(c->avg_bins.p, 0, sizeof(float2) * g * nbins, c->st));
  CK(cudaMemsetAsync(c->avg_count.p, 0, sizeof(int) * nbins, c->st));
  CK(cudaMemcpyAsync(c->avg_edges.p, npart_edges, sizeof(int) * (nbins + 1), cudaMemcpyHostToDevice, c->st));
  for (int off = 0; off < n; off += c->chunk) {
    const int m = std::min(c->chunk, n - off);
    CK(c->recs.ensure(m));
    CK(c->srcs.ensure((size_t)m * P.max_src));
    CK(c->status.ensure(m));
    CK(c->avg_rho.ensure((size_t)m * g));
    CK(c->ecc.ensure((size_t)m * smc::kEccLen));
    CK(c->avg_frame.ensure(m));
    CK(c->avg_order.ensure(m));
    if (method == 0) CK(c->avg_state.ensure((size_t)m * P.max_src));
    const int grid1 = std::max(1, std::min(m, c->sms * c->occ1));
    const int grid3 = std::max(1, std::min(m, c->sms * 4));
    auto splat = [&]() {
      return timed(c, 1, [&] {
        return launch_splat(c, P, m, c->recs.p, c->srcs.p, c->avg_rho.p, nullptr, nullptr, nullptr, c->ecc.p,
                            c->status.p);
      });
    };
    CK(timed(c, 0, [&] {
      return smc::launch_sample_pair(P, first_event + off, m, nullptr, nullptr, nullptr, c->recs.p, c->srcs.p,
                                     nullptr, nullptr, grid1, c->st);
    }));
    if (method == 0) CK(smc::launch_avg_init(P, m, c->recs.p, c->srcs.p, c->avg_state.p, grid3, c->st));
    CK(splat());
    // method 0: MCnucl::rotateGrid (src/MCnucl.cpp:1152-1174) and a second
    // splat; method 1: the frame only, the density is resampled below
    CK(smc::launch_avg_transform(P, m, c->recs.p, c->srcs.p, c->avg_state.p, c->avg_rho.p, order,
                                 method == 0 ? 1 : 2, grid3, c->st, c->avg_frame.p));
    if (method == 0) CK(splat());
    CK(smc::launch_avg_bins(c->recs.p, m, c->avg_edges.p, nbins, c->avg_order.p, c->avg_seg.p, c->avg_count.p,
                            c->st));
    CK(timed(c, 2, [&] {
      return smc::launch_avg_binned(P, c->recs.p, c->avg_rho.p, method == 1 ? c->avg_frame.p : nullptr, c->avg_order.p,
                                    c->avg_seg.p, nbins, c->avg_bins.p, slices > 1 ? c->avg_part.p : nullptr, c->st);
    }));
    c->stats.launches += method == 0 ? 3 : 2;
    c->h_status.resize(m);
    CK(cudaMemcpyAsync(c->h_status.data(), c->status.p, sizeof(int) * m, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    collect_timing(c);
    c->stats.events += m;
    int worst = 0;
    for (int e = 0; e < m; e++) worst = std::max(worst, c->h_status[e]);
    if (worst) return status_error(worst);
  }
  std::vector<float2> h(g * nbins);
  std::vector<int> cnt(nbins);
  CK(cudaMemcpyAsync(h.data(), c->avg_bins.p, sizeof(float2) * h.size(), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(cnt.data(), c->avg_count.p, sizeof(int) * nbins, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  // MakeDensity::setSd (src/MakeDensity.cpp:2514-2522): entropy = rho * finalFactor
  const double ff = c->P.final_factor;
  for (int b = 0; b < nbins; b++) {
    if (counts) counts[b] = cnt[b];
    for (size_t k = 0; k < g; k++) {
      const float2 a = h[(size_t)b * g + k];
      mean[(size_t)b * g + k] = cnt[b] ? ((double)a.x - (double)a.y) / cnt[b] * ff : 0.0;
    }
  }
  return SMC_OK;
}

// The launch sequence of a whole batch with device outputs and no host
// synchronisation: event ids from the device value ev_base, the worst
// event status reduced on the device and copied to h_worst at the end.
// Buffers must already have their sizes (no allocation: it is captured).
// The device buffers of the context that a captured batch reads or writes.
std::array<const void *, 12> batch_buffers(const Ctx *c) {
  return {c->recs.p, c->srcs.p, c->scratch.p, c->ecc.p, c->status.p, c->ev_order.p, c->tickets.p, c->corr_ev.p,
          c->rho_ev.p, c->cm_ev.p, c->ev_base.p, c->worst.p};
}

smc_status enqueue_batch(Ctx *c, int n, const smc_outputs *out, int *launches,
                         const smc::SystemDev *systems = nullptr, const int *ev_sys = nullptr,
                         const int *order = nullptr) {
  const DevParams &P = c->P;
  const size_t g = (size_t)P.nx * P.ny;
  const int AB = c->info.A + c->info.B;
  int nl = 0;
  CK(cudaMemcpyAsync(c->ev_base.p, c->h_first, sizeof(uint64_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(c->worst.p, 0, sizeof(int), c->st));
  for (int off = 0; off < n; off += c->chunk) {
    const int m = std::min(c->chunk, n - off);
    double *ecc = out->ecc ? out->ecc + (size_t)off * smc::kEccLen : c->ecc.p;
    float *rho = out->rho ? out->rho + (size_t)off * g : nullptr;
    float *ta = out->ta ? out->ta + (size_t)off * g : nullptr;
    float *tb = out->tb ? out->tb + (size_t)off * g : nullptr;
    double *pos = out->positions ? out->positions + (size_t)off * 2 * AB : nullptr;
    uint8_t *wnd = out->wounded ? out->wounded + (size_t)off * AB : nullptr;
    smc::TangentIO tio{};
    tio.ntan = out->tangents ? out->tangents + (size_t)off * 4 * AB : nullptr;
    tio.orient = out->orientation ? out->orientation + (size_t)off * 4 : nullptr;
    const int grid1 = std::max(1, std::min(m, c->sms * c->occ1));
    CK(smc::launch_sample_pair_mixed(P, off, m, nullptr, nullptr, nullptr, c->recs.p, c->srcs.p, pos, wnd, systems,
                                     ev_sys ? ev_sys + off : nullptr, order ? order + off : nullptr, grid1, c->st,
                                     &tio, c->ev_base.p, c->tickets.p + 2));
    CK(launch_splat(c, P, m, c->recs.p, c->srcs.p, rho, ta, tb, c->scratch.p, ecc, c->status.p));
    nl += 3 + ((c->use_tc && smc::grid_tc_supported(P) && !P.no_moments) ? 1 : 0);
    int *np = out->npart ? out->npart + 2 * off : nullptr;
    int *nc = out->ncoll ? out->ncoll + off : nullptr;
    double *bb = out->b ? out->b + off : nullptr;
    int *at = out->attempts ? out->attempts + off : nullptr;
    if (np || nc || bb || at) {
      k_scalars<<<(m + 255) / 256, 256, 0, c->st>>>(c->recs.p, m, np, nc, bb, at);
      CK(cudaGetLastError());
      nl++;
    }
    if (out->collisions) {
      k_collisions<<<(m + 7) / 8, 256, 0, c->st>>>(c->recs.p, c->srcs.p, m, P.max_src, P.max_coll,
                                                   out->collisions + (size_t)off * 2 * P.max_coll);
      CK(cudaGetLastError());
      nl++;
    }
    k_status_max<<<(m + 255) / 256, 256, 0, c->st>>>(c->status.p, m, c->worst.p);
    CK(cudaGetLastError());
    nl++;
  }
  CK(cudaMemcpyAsync(c->h_worst, c->worst.p, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  *launches = nl;
  return SMC_OK;
}

smc_status smc_autotune(void *ctx, int n_events, smc_tuning *out) {
  if (!ctx || n_events < 0) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  const int n = n_events > 0 ? n_events : 8192;
  CK(cudaSetDevice(c->device));
  smc_outputs none{};
  smc_status s = set_thickness_flags(c, &none);
  if (s) return s;
  DevBuf<double> ecc;
  CK(ecc.ensure((size_t)n * smc::kEccLen));
  smc_outputs o{};
  o.device = 1;
  o.ecc = ecc.p;
  const bool tc_ok = smc::grid_tc_supported(c->P);
  static const int chunks[4] = {2048, 4096, 8192, 16384};
  smc_tuning t{};
  double best = -1;
  const bool saved_timing = c->timing;
  c->timing = false;
  uint64_t first = (uint64_t)1 << 62;   // event ids of the trial batches
  for (int path = 1; path >= 0; path--) {
    for (int q = 0; q < 4; q++) {
      const int k = (1 - path) * 4 + q;
      t.events_per_s[k] = 0;
      if (path == 1 && !tc_ok) continue;
      c->use_tc = path == 1;
      c->chunk = chunks[q];
      s = run(c, first, std::min(n, chunks[q]), &o, nullptr, nullptr, nullptr, false);   // warm-up, buffers
      if (s && s != SMC_ERR_ZERO_DNDY) { ecc.release(); c->timing = saved_timing; return s; }
      first += n;
      const auto t0 = std::chrono::steady_clock::now();
      s = run(c, first, n, &o, nullptr, nullptr, nullptr, false);
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (s && s != SMC_ERR_ZERO_DNDY) { ecc.release(); c->timing = saved_timing; return s; }
      first += n;
      t.events_per_s[k] = n / dt;
      if (t.events_per_s[k] > best) {
        best = t.events_per_s[k];
        t.tensor_cores = path;
        t.chunk = chunks[q];
      }
    }
  }
  c->timing = saved_timing;
  c->use_tc = t.tensor_cores != 0;
  c->chunk = t.chunk;
  ecc.release();
  c->stats = smc_stats{};
  if (out) *out = t;
  return SMC_OK;
}

smc_status smc_generate_graph(void *ctx, uint64_t first_event, int n, const smc_outputs *out) {
  if (!ctx || !out || n < 0 || !out->device) return SMC_ERR_ARGUMENT;
  if (out->rho_pt || out->rho_binary || out->spectator_a || out->spectator_b) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  if (n == 0) return SMC_OK;
  CK(cudaSetDevice(c->device));
  smc_status s = set_thickness_flags(c, out);
  if (s) return s;
  const bool same = c->graph && c->graph_n == n && c->graph_chunk == c->chunk && c->graph_tc == c->use_tc &&
                    std::memcmp(&c->graph_out, out, sizeof(smc_outputs)) == 0 && c->graph_bufs == batch_buffers(c);
  if (!same) {
    // this call runs eagerly (sizing every buffer), then the batch is captured
    if (c->graph) {
      cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
    }
    s = run(c, first_event, n, out, nullptr, nullptr, nullptr, false);
    if (s && s != SMC_ERR_ZERO_DNDY) return s;
    CK(c->ev_base.ensure(1));
    CK(c->worst.ensure(1));
    if (!c->h_first) CK(cudaHostAlloc(&c->h_first, sizeof(uint64_t), cudaHostAllocDefault));
    if (!c->h_worst) CK(cudaHostAlloc(&c->h_worst, sizeof(int), cudaHostAllocDefault));
    CK(c->scratch.ensure((size_t)c->sms * c->occ2 * c->P.nx * c->P.ny));
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    int launches = 0;
    const bool timing = c->timing;
    c->timing = false;
    const smc_status se = enqueue_batch(c, n, out, &launches);
    c->timing = timing;
    const cudaError_t ee = cudaStreamEndCapture(c->st, &graph);
    if (se) {
      if (graph) cudaGraphDestroy(graph);
      return se;
    }
    CK(ee);
    const cudaError_t ei = cudaGraphInstantiate(&c->graph, graph, 0);
    cudaGraphDestroy(graph);
    CK(ei);
    c->graph_n = n;
    c->graph_chunk = c->chunk;
    c->graph_tc = c->use_tc;
    c->graph_out = *out;
    c->graph_launches = launches;
    c->graph_bufs = batch_buffers(c);
    return s;
  }
  *c->h_first = first_event;
  CK(cudaGraphLaunch(c->graph, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->stats.launches += c->graph_launches;
  c->stats.events += n;
  return status_error(*c->h_worst);
}

smc_status smc_generate_mixed_graph(void *ctx, const smc_params *systems, int nsys, uint64_t first_event, int n,
                                    const int *system_of_event, const smc_outputs *out) {
  if (!ctx || !out || n < 0 || !out->device) return SMC_ERR_ARGUMENT;
  if (out->rho_pt || out->rho_binary || out->spectator_a || out->spectator_b) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  if (n == 0) return SMC_OK;
  CK(cudaSetDevice(c->device));
  const bool same = c->mgraph && c->mgraph_n == n && c->mgraph_chunk == c->chunk && c->mgraph_tc == c->use_tc &&
                    std::memcmp(&c->mgraph_out, out, sizeof(smc_outputs)) == 0 && (int)c->mgraph_sys.size() == nsys &&
                    std::memcmp(c->mgraph_sys.data(), systems, sizeof(smc_params) * nsys) == 0 &&
                    std::memcmp(c->mgraph_ev.data(), system_of_event, sizeof(int) * n) == 0 &&
                    c->mgraph_bufs == batch_buffers(c);
  if (!same) {
    if (c->mgraph) {
      cudaGraphExecDestroy(c->mgraph);
      c->mgraph = nullptr;
    }
    // this call runs eagerly (checks the systems, sizes every buffer), then
    // the batch is captured with its own copies of the system table and of
    // each chunk's system list and event order
    smc_status s = smc_generate_mixed(ctx, systems, nsys, first_event, n, system_of_event, out);
    if (s && s != SMC_ERR_ZERO_DNDY) return s;
    std::vector<smc::SystemDev> sys;
    std::vector<int> cost, order, all_order(n);
    int max_ab = 0;
    smc_status v = mixed_systems(c, systems, nsys, n, system_of_event, out, sys, cost, max_ab);
    if (v) return v;
    for (int off = 0; off < n; off += c->chunk) {
      const int m = std::min(c->chunk, n - off);
      mixed_order(cost, system_of_event, off, m, order);
      std::copy(order.begin(), order.end(), all_order.begin() + off);
    }
    CK(c->mg_sys.ensure(nsys));
    CK(c->mg_ev.ensure(n));
    CK(c->mg_order.ensure(n));
    CK(cudaMemcpyAsync(c->mg_sys.p, sys.data(), sizeof(smc::SystemDev) * nsys, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->mg_ev.p, system_of_event, sizeof(int) * n, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->mg_order.p, all_order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->st));
    CK(c->ev_base.ensure(1));
    CK(c->worst.ensure(1));
    if (!c->h_first) CK(cudaHostAlloc(&c->h_first, sizeof(uint64_t), cudaHostAllocDefault));
    if (!c->h_worst) CK(cudaHostAlloc(&c->h_worst, sizeof(int), cudaHostAllocDefault));
    CK(c->scratch.ensure((size_t)c->sms * c->occ2 * c->P.nx * c->P.ny));
    CK(cudaStreamSynchronize(c->st));
    const int saved_max_src = c->P.max_src;
    c->P.max_src = 2 * max_ab + c->P.max_coll;   // as the eager call sized the sources
    cudaGraph_t graph = nullptr;
    const cudaError_t eb = cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal);
    int launches = 0;
    smc_status se = SMC_ERR_CUDA;
    cudaError_t ee = cudaErrorUnknown;
    if (eb == cudaSuccess) {
      const bool timing = c->timing;
      c->timing = false;
      se = enqueue_batch(c, n, out, &launches, c->mg_sys.p, c->mg_ev.p, c->mg_order.p);
      c->timing = timing;
      ee = cudaStreamEndCapture(c->st, &graph);
    }
    c->P.max_src = saved_max_src;
    if (eb != cudaSuccess) return SMC_ERR_CUDA;
    if (se) {
      if (graph) cudaGraphDestroy(graph);
      return se;
    }
    CK(ee);
    const cudaError_t ei = cudaGraphInstantiate(&c->mgraph, graph, 0);
    cudaGraphDestroy(graph);
    CK(ei);
    c->mgraph_n = n;
    c->mgraph_chunk = c->chunk;
    c->mgraph_tc = c->use_tc;
    c->mgraph_out = *out;
    c->mgraph_sys.assign(systems, systems + nsys);
    c->mgraph_ev.assign(system_of_event, system_of_event + n);
    c->mgraph_launches = launches;
    c->mgraph_bufs = batch_buffers(c);
    return s;
  }
  *c->h_first = first_event;
  CK(cudaGraphLaunch(c->mgraph, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->stats.launches += c->mgraph_launches;
  c->stats.events += n;
  return status_error(*c->h_worst);
}

smc_status smc_sample_nuclei(void *ctx, uint64_t event, double b, double *xy_proj, double *xy_targ, int *npart,
                             int *ncoll, double *orientation) {
  if (!ctx || !xy_proj || !xy_targ) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  CK(cudaSetDevice(c->device));
  const int A = c->info.A, B = c->info.B;
  CK(c->recs.ensure(1));
  CK(c->srcs.ensure(c->P.max_src));
  CK(c->pos.ensure((size_t)2 * (A + B)));
  CK(c->inj_b.ensure(1));
  CK(cudaMemcpyAsync(c->inj_b.p, &b, sizeof(double), cudaMemcpyHostToDevice, c->st));
  // one attempt at the given b, no centrality cut: an event without a
  // collision ends with the retry status after its first attempt
  DevParams P = c->P;
  P.max_attempts = 1;
  P.npmin = 0;
  P.npmax = 1 << 30;
  CK(smc::launch_sample_pair_mixed(P, event, 1, nullptr, nullptr, c->inj_b.p, c->recs.p, c->srcs.p, c->pos.p,
                                   nullptr, nullptr, nullptr, nullptr, 1, c->st));
  std::vector<double> pos((size_t)2 * (A + B));
  EventRec r{};
  CK(cudaMemcpyAsync(pos.data(), c->pos.p, sizeof(double) * pos.size(), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(&r, c->recs.p, sizeof(EventRec), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (r.status != 0 && r.status != 3) return status_error(r.status);
  std::copy(pos.begin(), pos.begin() + 2 * A, xy_proj);
  std::copy(pos.begin() + 2 * A, pos.end(), xy_targ);
  if (npart) { npart[0] = r.npart1; npart[1] = r.npart2; }
  if (ncoll) *ncoll = r.ncoll;
  if (orientation) {
    // the attempt's orientations, as the sampler draws them (whether or not
    // the event has a collision)
    for (int w = 0; w < 2; w++) {
      double o[2];
      smc::uniform2(c->P.seed, event, smc::stream_id(0, smc::ST_EVENT), 1 + w, o[0], o[1]);
      orientation[2 * w] = 1.0 - 2.0 * o[0];
      orientation[2 * w + 1] = 2 * M_PI * o[1];
    }
  }
  return SMC_OK;
}

smc_status smc_set_configurations(void *ctx, int A, const double *xyz, int nconf) {
  if (!ctx || A < 3 || A > smc::kMaxA || nconf < 0 || (nconf > 0 && !xyz)) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  const size_t cnt = (size_t)nconf * A * 3;
  for (size_t k = 0; k < cnt; k++)
    if (!std::isfinite(xyz[k])) return SMC_ERR_ARGUMENT;
  CK(cudaSetDevice(c->device));
  // the work queued on the old table ends before it is replaced
  CK(cudaStreamSynchronize(c->st));
  Ctx::ConfTab &t = c->conf[A];
  if (nconf == 0) {
    t.xyz.release();
    t.n = 0;
  } else {
    if (t.xyz.n < cnt) t.xyz.release();   // no stale table if the allocation fails
    t.n = 0;
    CK(t.xyz.ensure(cnt));
    CK(cudaMemcpy(t.xyz.p, xyz, sizeof(double) * cnt, cudaMemcpyHostToDevice));
    t.n = nconf;
  }
  attach_configurations(c, c->P.nuc[0]);
  attach_configurations(c, c->P.nuc[1]);
  // captured batches hold the old parameters
  if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  if (c->mgraph) { cudaGraphExecDestroy(c->mgraph); c->mgraph = nullptr; }
  return SMC_OK;
}

smc_status smc_read_configurations(int A, const char *path, double *xyz, int capacity, int *nconf) {
  if (!path || !nconf || A < 3 || A > smc::kMaxA || capacity < 0 || (capacity > 0 && !xyz))
    return SMC_ERR_ARGUMENT;
  *nconf = 0;
  std::ifstream in(path);
  if (!in.is_open()) return SMC_ERR_ARGUMENT;
  // the reference's record layouts (src/Nucleus.cpp:383-478): fields before
  // and after the 3 A coordinates of one configuration
  const int lead = A == 12 ? 2 : 0, trail = A == 3 ? 4 : 0;
  std::vector<double> rec((size_t)3 * A);
  int n = 0;
  for (;;) {
    double v;
    int got = 0;
    for (int k = 0; k < lead && (in >> v); k++) got++;
    for (int k = 0; k < 3 * A && (in >> rec[k]); k++) got++;
    for (int k = 0; k < trail && (in >> v); k++) got++;
    if (got == 0 && in.eof()) break;
    if (got != lead + 3 * A + trail) return SMC_ERR_ARGUMENT;   // a record cut short, or not a number
    if (n < capacity) std::copy(rec.begin(), rec.end(), xyz + (size_t)n * 3 * A);
    if (n == INT_MAX) return SMC_ERR_ARGUMENT;
    n++;
  }
  *nconf = n;
  if (n == 0) return SMC_ERR_ARGUMENT;
  return n > capacity ? SMC_ERR_CAPACITY : SMC_OK;
}

smc_status smc_load_configurations(void *ctx, int A, const char *path) {
  if (!ctx) return SMC_ERR_ARGUMENT;
  int n = 0;
  smc_status s = smc_read_configurations(A, path, nullptr, 0, &n);
  if (s != SMC_OK && s != SMC_ERR_CAPACITY) return s;
  std::vector<double> xyz((size_t)n * 3 * A);
  s = smc_read_configurations(A, path, xyz.data(), n, &n);
  if (s) return s;
  return smc_set_configurations(ctx, A, xyz.data(), n);
}

smc_status smc_set_grid_path(void *ctx, int tensor_cores) {
  if (!ctx) return SMC_ERR_ARGUMENT;
  static_cast<Ctx *>(ctx)->use_tc = tensor_cores != 0;
  return SMC_OK;
}

smc_status smc_set_timing(void *ctx, int enabled) {
  if (!ctx) return SMC_ERR_ARGUMENT;
  static_cast<Ctx *>(ctx)->timing = enabled != 0;
  return SMC_OK;
}

smc_status smc_get_stats(void *ctx, smc_stats *stats) {
  if (!ctx || !stats) return SMC_ERR_ARGUMENT;
  *stats = static_cast<Ctx *>(ctx)->stats;
  return SMC_OK;
}

smc_status smc_reset_stats(void *ctx) {
  if (!ctx) return SMC_ERR_ARGUMENT;
  static_cast<Ctx *>(ctx)->stats = smc_stats{};
  return SMC_OK;
}

smc_status smc_kln_table(void *ctx, double *host_table, int capacity) {
  if (!ctx || !host_table) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  if (c->P.which_mc_model != 1 || !c->kln64.p) return SMC_ERR_CONFIG;
  size_t n = (size_t)c->info.kln_tmax * c->info.kln_tmax;
  if ((size_t)capacity < n) return SMC_ERR_ARGUMENT;
  CK(cudaMemcpyAsync(host_table, c->kln64.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SMC_OK;
}

smc_status smc_kln_pt_table(void *ctx, double pt_min, double d_pt, int nbins, double *host_table, size_t capacity) {
  if (!ctx || nbins < 1 || nbins > 4096 || !(d_pt > 0) || !(pt_min > 0)) return SMC_ERR_ARGUMENT;
  Ctx *c = static_cast<Ctx *>(ctx);
  if (c->P.which_mc_model != 1 || !c->kln64.p) return SMC_ERR_CONFIG;
  const int tmax = c->info.kln_tmax;
  const size_t n = (size_t)tmax * tmax * nbins;
  if (host_table && capacity < n) return SMC_ERR_ARGUMENT;
  CK(cudaSetDevice(c->device));
  if (c->pt_nbins != nbins || c->pt_min != pt_min || c->pt_step != d_pt) {
    smc::KlnDev K;
    double *d_nodes = nullptr;
    smc_status s = kln_quadrature(c, K, &d_nodes);
    cudaError_t e = s ? cudaSuccess : c->pt64.ensure(n);
    if (!s && e == cudaSuccess) e = c->pt32.ensure(n);
    if (!s && e == cudaSuccess)
      e = smc::launch_kln_pt_table(K, tmax, c->info.kln_dT, pt_min, d_pt, nbins, c->pt64.p, c->pt32.p, c->st);
    if (!s && e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (d_nodes) cudaFree(d_nodes);
    if (s) return s;
    if (e != cudaSuccess) {
      c->pt_nbins = 0;
      return SMC_ERR_CUDA;
    }
    c->pt_nbins = nbins;
    c->pt_min = pt_min;
    c->pt_step = d_pt;
  }
  if (host_table) {
    CK(cudaMemcpyAsync(host_table, c->pt64.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  return SMC_OK;
}

}  // extern "C"
