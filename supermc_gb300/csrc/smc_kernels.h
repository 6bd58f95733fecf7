// Launchers of the sm_103a kernels (one translation unit each).
#pragma once
#include "smc_device.cuh"

namespace smc {

// MC-KLN quadrature description (KLNModel::func, src/KLNModel.cpp:219-277)
struct KlnDev {
  double ecm, lambda, y, ptmin, ptmax, lambda_qcd2, alpha_max, beta0, fac, prefactor;
  int npt, nkt, nphi;
  const double *xp, *wp, *xk, *wk, *xf, *wf;   // Gauss-Legendre nodes on [0,1]
  const double *cf;                            // cos(2 pi xf[f]), f <= nphi / 2
};

size_t sample_pair_smem();
cudaError_t launch_sample_pair(const DevParams &P, uint64_t first_event, int n_events, const double *inj_proj,
                               const double *inj_targ, const double *inj_b, EventRec *recs, Source *srcs,
                               double *out_pos, uint8_t *out_wounded, int grid, cudaStream_t st);
// Mixed batch: event e takes the system parameters systems[ev_sys[e]]; the
// CTAs take the events in the given order (NULL: 0, 1, ...).
// event ids are first_event + e, plus *ev_base when ev_base is given (a
// device value, so that a captured graph replays with new event ids)
cudaError_t launch_sample_pair_mixed(const DevParams &P, uint64_t first_event, int n_events, const double *inj_proj,
                                     const double *inj_targ, const double *inj_b, EventRec *recs, Source *srcs,
                                     double *out_pos, uint8_t *out_wounded, const SystemDev *systems,
                                     const int *ev_sys, const int *order, int grid, cudaStream_t st,
                                     const TangentIO *tio = nullptr, const uint64_t *ev_base = nullptr,
                                     int *ticket = nullptr);
size_t grid_smem(const DevParams &P);
int grid_blocks_per_sm(const DevParams &P);
// the grid kernels take their events from a queue (EventQueue): with ticket
// (a device counter the launcher zeroes) dynamically, in `order` when given
cudaError_t launch_grid(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs, float *out_rho,
                        float *out_ta, float *out_tb, float *scratch, double *out_ecc, int *status, int grid,
                        cudaStream_t st, const int *order = nullptr, int *ticket = nullptr);
size_t grid_tc_smem(const DevParams &P);
bool grid_tc_supported(const DevParams &P);
// Tensor-core splat of a batch: contraction, corner corrections and post-op
// (k_grid_tc, one CTA per SM), then the eccentricities (k_moments, unless
// P.no_moments).  Buffers: rho_ev [n][nx][ny] floats (the densities when
// out_rho is NULL), corr_scratch [sms][n_planes][nx][ny] ints (per-CTA
// corner corrections), cm_ev [n][3] doubles (centre-of-mass sums).
cudaError_t launch_grid_tc(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs,
                           float *out_rho, float *out_ta, float *out_tb, float *rho_ev, int *corr_scratch,
                           double *cm_ev, double *out_ecc, int *status, int sms, cudaStream_t st,
                           const int *order = nullptr, int *tickets = nullptr);
cudaError_t launch_avg_init(const DevParams &P, int n, const EventRec *recs, const Source *srcs, AvgSrc *state,
                            int grid, cudaStream_t st);
cudaError_t launch_avg_transform(const DevParams &P, int n, EventRec *recs, Source *srcs, AvgSrc *state,
                                 const float *rho, int order, int mode, int grid, cudaStream_t st,
                                 AvgFrame *frame = nullptr);
// centrality bins of a chunk (order[], seg[nbins + 1], counts[nbins] +=)
cudaError_t launch_avg_bins(const EventRec *recs, int n, const int *edges, int nbins, int *order, int *seg,
                            int *counts, cudaStream_t st);
// per-bin compensated sums acc [nbins][nx][ny] of the chunk's densities,
// bilinearly resampled in each event's frame (frame != NULL) or as they are;
// part (else NULL: one slice): scratch of avg_binned_slices(P) x nbins x
// nx x ny float2 for the event slices of each bin, merged in order
int avg_binned_slices(const DevParams &P);
cudaError_t launch_avg_binned(const DevParams &P, const EventRec *recs, const float *rho, const AvgFrame *frame,
                              const int *order, const int *seg, int nbins, float2 *acc, float2 *part,
                              cudaStream_t st);
cudaError_t launch_avg_accum(const float *rho, int n, size_t cells, double *acc, cudaStream_t st);
// averaged mode's derived grids: source views (0: rho_binary, 1: spectators)
// and the T_A T_B product accumulation
cudaError_t launch_avg_view(const DevParams &P, int n, const EventRec *recs, const Source *in, Source *out, int mode,
                            EventRec *vrecs, int grid, cudaStream_t st);
cudaError_t launch_avg_accum_prod(const float *a, const float *b, int n, size_t cells, double *acc, cudaStream_t st);
// Adjoint of a batch (k_adjoint, one CTA per event in turn): per-event
// gradients dtheta [n][4] = (dL/dw, dL/dalpha, dL/dR, dL/da; the last two
// through the source position tangents src_tan [n][max_src], zero when
// src_tan is NULL) of
// L = sum_e g_eps[e][0] |eps_2| + g_eps[e][1] |eps_3| + <g_rho[e], rho_e>
// from the forward densities rho_ev [n][nx][ny]; g_eps, g_rho may be NULL;
// lam_scratch [grid][nx][ny] floats.
size_t adjoint_smem(const DevParams &P);
int adjoint_blocks_per_sm(const DevParams &P);
cudaError_t launch_adjoint(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs,
                           const float4 *src_tan, const float *rho_ev, const float *g_grid, const double *g_eps,
                           float *lam_scratch, double *dtheta, int grid, cudaStream_t st, const int *order = nullptr,
                           int *ticket = nullptr);
cudaError_t launch_kln_table(const KlnDev &K, int tmax, double dT, double *table64, float *table32,
                             cudaStream_t st);
// p_T-differential table [tmax][tmax][nbins] (k_kln_pt_table)
cudaError_t launch_kln_pt_table(const KlnDev &K, int tmax, double dT, double ptmin, double dpt, int nbins,
                                double *table64, float *table32, cudaStream_t st);
// per-cell p_T-differential densities out [n][nx][ny][nbins] from the
// events' thickness grids ta, tb [n][nx][ny] and the FP32 table
cudaError_t launch_kln_pt_cells(const DevParams &P, int n, const EventRec *recs, const Source *srcs, const float *ta,
                                const float *tb, const float *table, int nbins, float *out, int *status, int grid,
                                cudaStream_t st);

}  // namespace smc
