/* supermc_gb300 -- C ABI of the GB300 (sm_103a) initial-condition engine.
 *
 * Drop-in boundary for superMC's per-event path.  In the reference the path
 * sits behind two C++ classes called from main() (src/main.cpp:35-61):
 *   MakeDensity(ParameterReader*)               src/MakeDensity.h:43
 *     generateEccTable / generate_profile_ebe / generate_profile_average /
 *     dumpEccentricities                         src/MakeDensity.h:53-57
 *   MCnucl(ParameterReader*)                    src/MCnucl.h:87
 *     generateNuclei, getBinaryCollision, CentralityCut, calculateThickness,
 *     setDensity, getTA1/getTA2/getRho, rotateGrid, makeTable
 *                                               src/MCnucl.h:94-130
 * Each entry point below names the reference call(s) it replaces.  All
 * functions return an smc_status; none calls exit() (the reference exits on
 * a missing parameter, a zero dN/dy or a KLN table overflow,
 * src/ParameterReader.cpp:195, src/MCnucl.cpp:812-816, :665-670).
 *
 * Threading: one context per host thread at a time; calls on one context
 * are serialised on the context's CUDA stream.  Host pointers are borrowed
 * for the duration of the call.  Device buffers are owned by the context.
 */
#ifndef SUPERMC_GB300_H
#define SUPERMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int smc_status;
enum {
  SMC_OK = 0,
  SMC_ERR_ARGUMENT = 1,     /* bad pointer / size / order range            */
  SMC_ERR_CONFIG = 2,       /* unsupported or inconsistent parameters       */
  SMC_ERR_RETRY_CAP = 3,    /* event retry loop hit its cap (reference loops
                               forever, src/MakeDensity.cpp:2147-2162)      */
  SMC_ERR_KLN_TABLE = 4,    /* thickness beyond the dN/dy table
                               (src/MCnucl.cpp:424-428, :665-670)           */
  SMC_ERR_ZERO_DNDY = 5,    /* integrated density is zero (MCnucl.cpp:812)  */
  SMC_ERR_CAPACITY = 6,     /* a per-event buffer (collisions) overflowed   */
  SMC_ERR_CUDA = 7,         /* CUDA runtime error                           */
  SMC_ERR_NO_DEVICE = 8,    /* no usable GPU                                */
  SMC_ERR_SCRATCH_LIMIT = 9 /* request larger than smc_inject_noalloc's
                               fixed scratch                                */
};

/* Physics and grid configuration: the parameters.dat keys of the path
 * (reference parameters.dat, read by src/ParameterReader.cpp), plus
 * optional overrides for values the reference hard-codes (<= 0 keeps the
 * reference value). */
typedef struct smc_params {
  int which_mc_model;       /* 5 = MC-Glauber, 1 = MC-KLN, 7 = sqrt(T_A T_B)  */
  int sub_model;            /* Glauber: 1 classical, 2 Heinz-Qiu-Moreland;
                               KLN: 7                                        */
  int shape_of_nucleons;    /* 1 disk, 2 Gaussian from sigma, 4 user width  */
  int shape_of_entropy;     /* 1 disk, 2 Gaussian                           */
  int collision_criterion;  /* 1 disk (d^2 <= sigma/pi), 2 Gaussian profile */
  int Aproj, Atarg;         /* mass numbers (1 = p, 2 = d, else Woods-Saxon
                               or a configuration table:
                               smc_set_configurations)                     */
  int proj_deformed, targ_deformed;
  double ecm;               /* sqrt(s) [GeV]; sigma_in from Regge fits      */
  double alpha;             /* (1-alpha)/2 WN + alpha BC                    */
  double gauss_nucl_width;  /* width for shape_of_nucleons = 4 [fm]        */
  double quark_width;       /* valence-quark box width [fm]                 */
  double lambda;            /* KLN saturation exponent                      */
  double bmin, bmax;        /* impact-parameter range [fm]                  */
  int npmin, npmax;         /* Npart acceptance                             */
  double maxx, maxy, dx, dy;/* grid half-width and spacing [fm]             */
  double final_factor;      /* finalFactor                                  */
  int tmax, tmax_subdivision; /* KLN dN/dy table size                       */
  int ecc_from_order, ecc_to_order;
  /* extensions (<= 0: reference value) */
  double proj_R, proj_a, targ_R, targ_a; /* Woods-Saxon radius/diffuseness  */
  double proj_d_min, targ_d_min;         /* hard-core distance              */
  double sigin_override;                 /* sigma_in [mb]                   */
  int kln_npt, kln_nkt, kln_nphi;        /* KLN table quadrature nodes      */
  uint64_t seed;                         /* Philox key                      */
  int max_attempts;                      /* event retry cap (0: 100000)     */
  int max_collisions;                    /* per-event collision capacity
                                            (0: 4096)                       */
  int ws_inverse_cdf;                    /* 1: Woods-Saxon radii by inverse
                                            CDF of the reference's truncated
                                            density (r <= R + 2.5) instead of
                                            rejection, so that positions are
                                            differentiable in R and a
                                            (smc_adjoint); spherical A > 2 */
  int cc_fluctuation_model;              /* 0 none; 6: mean-one Gamma weight per
                                            participant and binary collision
                                            (MCnucl.cpp:1271-1301; the
                                            reference's parameters.dat default);
                                            1, 2: per-cell negative-binomial
                                            density (MCnucl::fluctuateCurrent-
                                            Density, :869-905) with k =
                                            cc_fluctuation_k (1) or from
                                            min(T_A, T_B) (2); 3-5 rejected */
  double cc_fluctuation_gamma_theta;     /* Gamma scale (cc_fluctuation_Gamma_theta) */
  double cc_fluctuation_k;               /* NBD shape of model 1 (cc_fluctuation_k)  */
  double kln_exact_band;                 /* MC-KLN: the per-cell table cell
                                            floor(T/dT) (src/MCnucl.cpp:659-
                                            670) is taken from FP64 thickness
                                            sums where T/dT lies within this
                                            relative distance of an integer
                                            (<= 0: the error bound of the FP32
                                            sums, so every cell is decided as
                                            in FP64; larger values only move
                                            more cells to the FP64 path)    */
} smc_params;

/* Derived constants (MCnucl::MCnucl, src/MCnucl.cpp:22-154). */
typedef struct smc_info {
  int nx, ny;               /* Maxx, Maxy                                   */
  double sigin;             /* inelastic NN cross section [mb]              */
  double dsq;               /* 0.1 sigma_in / pi [fm^2]                     */
  double width;             /* nucleon width [fm]                           */
  double sigma_gg;          /* Gaussian-profile cross section [fm^2]        */
  int kln_tmax;             /* subdivided table size                        */
  double kln_dT;            /* table thickness step [fm^-2]                 */
  int A, B;                 /* nucleons per nucleus                         */
  int max_collisions;       /* per-event collision capacity (rows of
                               smc_outputs.collisions)                      */
} smc_info;

/* Per-event results.  Every pointer may be NULL (not produced).  When
 * `device` is non-zero the pointers are device memory of the context's GPU,
 * otherwise host memory (copied back inside the call). */
typedef struct smc_outputs {
  int device;
  double *ecc;          /* [n][49]: orders 1..9 x (Re,Im r^2-weighted,
                           Re,Im r^n-weighted, <r^n>), Npart, Ncoll,
                           integral rho*finalFactor*dx*dy, b -- the line
                           MakeDensity::dumpEccentricities appends to
                           sn_ecc_eccp_10.dat (src/MakeDensity.cpp:2473-2500) */
  float *rho;           /* [n][nx][ny] density (MCnucl::getRho)              */
  float *ta, *tb;       /* [n][nx][ny] thickness (MCnucl::getTA1/getTA2)     */
  int *npart;           /* [n][2] Npart1, Npart2                             */
  int *ncoll;           /* [n]                                               */
  double *b;            /* [n] impact parameter                              */
  int *attempts;        /* [n] tries per accepted event                      */
  double *positions;    /* [n][A+B][2] nucleon x,y (projectile first, each
                           nucleus sorted by x)                              */
  uint8_t *wounded;     /* [n][A+B] 1 = participant                          */
  double *tangents;     /* [n][A+B][4] d(x,y)/dR, d(x,y)/da of each nucleon
                           (same order as positions; both nuclei's R, a
                           move together; zero unless ws_inverse_cdf)        */
  double *collisions;   /* [n][max_collisions][2] binary-collision positions
                           (pair midpoints) in the reference's order
                           (MCnucl::createBinaryCollisions, src/MCnucl.cpp:
                           326-352); the first ncoll rows of each event     */
  double *orientation;  /* [n][4] cos(theta), phi of the projectile, then of
                           the target: the orientation Nucleus::populate
                           draws for the accepted attempt (src/Nucleus.cpp:
                           192-197; it rotates deformed nuclei); zero for
                           injected nuclei.  The deformed layout of the
                           eccentricity files carries it
                           (smc_write_ecc_deformed)                          */
  /* The fields below are not produced by the graph-captured batches
   * (smc_generate_graph, smc_generate_mixed_graph: SMC_ERR_ARGUMENT). */
  float *rho_pt;        /* [n][nx][ny][nbins] MC-KLN p_T-differential dN/dy
                           d^2p_T per cell (MCnucl::setDensity(iy, ipt) for
                           every bin, src/MCnucl.cpp:626-687, getRho(iy, i,
                           j, ipt)); needs smc_kln_pt_table first (nbins are
                           its bins; ignored before it)                      */
  float *rho_binary;    /* [n][nx][ny] binary-collision density
                           (MCnucl::calculate_rho_binary, src/MCnucl.cpp:
                           481-531): a unit-normalised Gaussian (or disk) per
                           collision, r <= 5w                                */
  float *spectator_a, *spectator_b;   /* [n][nx][ny] spectator densities of
                           the projectile and the target
                           (MCnucl::calculate_spectator_density, :534-614)   */
} smc_outputs;

/* MCnucl::MCnucl + MakeDensity::MakeDensity: validates the configuration,
 * selects device 0 of the process, allocates device state.  For
 * which_mc_model = 1 the dN/dy table is built on the GPU here
 * (MCnucl::makeTable, src/MCnucl.cpp:911-960). */
smc_status smc_create(const smc_params *params, void **ctx_out);
void smc_destroy(void *ctx);
smc_status smc_get_info(void *ctx, smc_info *info);
const char *smc_status_string(smc_status s);
/* Name and description of the calling thread's last CUDA runtime error, for
 * the message of an SMC_ERR_CUDA status (cudaGetLastError: reading it clears
 * an error that is not sticky; "cudaSuccess: no error" when none is pending).
 * The string lives until the thread's next call. */
const char *smc_cuda_error_string(void);
/* Runs subsequent work on the given cudaStream_t (NULL: the context's own
 * stream). */
smc_status smc_set_stream(void *ctx, void *cuda_stream);
smc_status smc_synchronize(void *ctx);

/* Event generation, one batch: the event loop of
 * MakeDensity::generateEccTable / generate_profile_ebe
 * (src/MakeDensity.cpp:2143-2196, :574-694) for events
 * [first_event, first_event + n).  Each event draws its impact parameter
 * and nuclei (MCnucl::generateNuclei, Nucleus::populate) from Philox
 * streams keyed by (seed, event id), retries until Ncoll > 0 and
 * npmin <= Npart <= npmax (MCnucl::getBinaryCollision, CentralityCut),
 * then computes thickness, density (MCnucl::calculateThickness,
 * setDensity) and eccentricities (MakeDensity::dumpEccentricities). */
smc_status smc_generate(void *ctx, uint64_t first_event, int n, const smc_outputs *out);

/* The same pipeline from given nucleon positions (the reference's injection
 * harness path): xy_proj [n][A][2], xy_targ [n][B][2], b [n] (may be NULL),
 * host memory unless out->device.  Replaces getBinaryCollision +
 * calculateThickness + setDensity + dumpEccentricities on injected
 * nuclei. */
smc_status smc_inject(void *ctx, int n, const double *xy_proj, const double *xy_targ,
                      const double *b, const smc_outputs *out);

/* Mixed-system batch: events of several collision systems in one launch
 * per stage (the reference runs one system per process, src/main.cpp:35-61,
 * so a mixed sample there is several runs).  systems[0..nsys) are full
 * parameter sets that may differ from the context's only in Aproj, Atarg,
 * the deformation flags, ecm / sigin_override, the Woods-Saxon and hard-core
 * overrides, bmin, bmax, npmin and npmax; everything else (model, nucleon
 * and entropy shape -- shape_of_nucleons 4 --, grid, alpha, orders, seed)
 * must equal the context's.  Event first_event + e belongs to system
 * system_of_event[e] and draws the Philox streams it would draw in a
 * single-system context of that system, so its results are the same.
 * Within each chunk the heavier systems are scheduled first.  MC-Glauber
 * and sqrt(T_A T_B) only (MC-KLN tables are per energy); out->positions and
 * out->wounded are not produced (their shapes differ between systems). */
smc_status smc_generate_mixed(void *ctx, const smc_params *systems, int nsys, uint64_t first_event, int n,
                              const int *system_of_event, const smc_outputs *out);

/* smc_generate as one CUDA graph: the launch sequence of the whole batch
 * (every chunk's sampling, splat and eccentricity kernels, the per-event
 * status reduced on the device, no host synchronisation in between) is
 * captured on the first call for a given n, output set and launch
 * configuration -- that call runs eagerly -- and replayed by later calls
 * with new event ids (an on-device event-id base).  Device outputs only
 * (out->device != 0); the results equal smc_generate's. */
smc_status smc_generate_graph(void *ctx, uint64_t first_event, int n, const smc_outputs *out);

/* smc_generate_mixed as one CUDA graph: the whole mixed batch (every
 * chunk's sampling with its systems and heavy-systems-first order, splat,
 * eccentricities and the device-side status reduction) is captured on the
 * first call for a given n, system table, per-event systems, output set and
 * launch configuration -- that call runs eagerly -- and replayed by later
 * calls with new event ids.  Device outputs only (out->device != 0); the
 * results equal smc_generate_mixed's.  The reference runs one system per
 * process (src/main.cpp:35-61); no counterpart. */
smc_status smc_generate_mixed_graph(void *ctx, const smc_params *systems, int nsys, uint64_t first_event, int n,
                                    const int *system_of_event, const smc_outputs *out);

/* MCnucl::generateNuclei(b) + getBinaryCollision (src/MCnucl.cpp:208-308)
 * for one event: both nuclei drawn from the Philox streams of (seed,
 * event) at the given impact parameter, then paired (one attempt, no
 * centrality cut, no retry).  xy_proj [A][2], xy_targ [B][2] (host) receive
 * the nucleons (each nucleus sorted by x), npart [2] Npart1, Npart2, *ncoll
 * the binary collisions (0: none), orientation [4] cos(theta), phi of each
 * nucleus (Nucleus::populate, src/Nucleus.cpp:192-197); npart, ncoll and
 * orientation may be NULL.  The nuclei then go through smc_inject. */
smc_status smc_sample_nuclei(void *ctx, uint64_t event, double b, double *xy_proj, double *xy_targ, int *npart,
                             int *ncoll, double *orientation);

/* Light-nucleus configurations (Nucleus::readin_helium3_position ..
 * readin_oxygen_position and GetNucleonPosition, src/Nucleus.cpp:383-478,
 * 555-574): every nucleus of mass number A (3 <= A <= 256) of this
 * context -- projectile, target, the systems of a mixed batch -- takes one
 * configuration of xyz [nconf][A][3] (nucleus-frame x, y, z in fm, host
 * memory) per event instead of Woods-Saxon sampling: configuration
 * floor(u nconf) with u from the event's Philox stream 7 (the reference:
 * rand() % nconf), rotated by the nucleus orientation (Point3D::rotate),
 * shifted by +-b/2 and not recentred (src/Nucleus.cpp:210-236).
 * nconf = 0 removes A's table.  Non-finite positions: SMC_ERR_ARGUMENT.
 * The table is copied to the device; captured graphs are re-captured. */
smc_status smc_set_configurations(void *ctx, int A, const double *xyz, int nconf);

/* The light-nucleus configuration files in the reference's layout for A
 * (one configuration per record, whitespace-separated fields): A = 3
 * (tables/he3_plaintext.dat): 9 coordinates and 4 further fields; A = 12
 * (tables/carbon_plaintext.dat): 2 fields and 36 coordinates; any other A
 * (tables/he4_plaintext.dat, tables/oxygen_plaintext.dat): 3 A coordinates.
 * Records are read until the file ends.  smc_read_configurations needs no
 * GPU: *nconf receives the file's configuration count and xyz [capacity][A][3]
 * the first capacity of them (SMC_ERR_CAPACITY when more are in the file;
 * xyz may be NULL with capacity 0 to count).  A file that cannot be opened,
 * holds no complete record or ends inside one: SMC_ERR_ARGUMENT.
 * smc_load_configurations reads a file and passes it to
 * smc_set_configurations. */
smc_status smc_read_configurations(int A, const char *path, double *xyz, int capacity, int *nconf);
smc_status smc_load_configurations(void *ctx, int A, const char *path);

/* Plain per-event path: the same results as smc_generate, one event per
 * kernel launch sequence (the unbatched baseline). */
smc_status smc_generate_plain(void *ctx, uint64_t first_event, int n, const smc_outputs *out);

/* Averaged profiles: MakeDensity::generate_profile_average
 * (src/MakeDensity.cpp:736-2103, per-event loop :1240-1577).  For events
 * [first_event, first_event + n) -- generated, or injected when xy_proj /
 * xy_targ (host, [n][A][2], [n][B][2]) are given -- and every order
 * n_ord = from_order..to_order in turn, the sources are rotated to the
 * order-n_ord participant plane about the density's centre of mass
 * (MCnucl::rotateGrid, src/MCnucl.cpp:1152-1174) and re-splatted; with
 * reaction_plane != 0 they are first recentred only
 * (MCnucl::recenterGrid, :1119-1150; the reaction-plane-frame average).
 * mean / mean_rp [to-from+1][nx][ny] (host) receive the event averages of
 * the entropy density getRho * finalFactor (MakeDensity::setSd,
 * :2514-2522) over the events with a binary collision (their count in
 * *n_used, may be NULL; injected events without one are left out).  The
 * moves accumulate across orders as in the reference. */
smc_status smc_average(void *ctx, uint64_t first_event, int n, const double *xy_proj,
                       const double *xy_targ, const double *b, int from_order, int to_order,
                       int reaction_plane, double *mean, double *mean_rp, int *n_used);

/* All averaged profiles of MakeDensity::generate_profile_average
 * (src/MakeDensity.cpp:1240-1577) for the integrated-p_T entropy density:
 * for every order from_order..to_order and both frames -- the
 * participant plane (rotateGrid) and the reaction plane (recenterGrid, the
 * *_rp grids) -- the event means, after each frame's transform, of
 *   sd          rho * finalFactor           (sdAvg[_RP]_order_<n>)
 *   ta_tb       T_A T_B                     (TATB_fromSd[_RP]_order_<n>, :1342-1349)
 *   ta, tb      T_A, T_B                    (nuclear_thickness_T{A,B}_fromSd[_RP]_order_<n>, :1362-1370)
 *   rho_binary  unit Gaussians at the binary collisions
 *               (MCnucl::calculate_rho_binary, src/MCnucl.cpp:481-531)
 *   spectator_a/_b  unit Gaussians at the projectile / target spectators
 *               (MCnucl::calculate_spectator_density, :534-614)
 * Each pointer is host memory [to-from+1][nx][ny] or NULL (not produced;
 * the reaction-plane frame runs when any *_rp pointer is set).  Events and
 * moves as for smc_average; T_A T_B and the thickness means need
 * which_mc_model 5 or 1. */
typedef struct smc_average_outputs {
  double *sd, *sd_rp;
  double *ta_tb, *ta_tb_rp;
  double *ta, *tb, *ta_rp, *tb_rp;
  double *rho_binary, *rho_binary_rp;
  double *spectator_a, *spectator_b, *spectator_a_rp, *spectator_b_rp;
} smc_average_outputs;
smc_status smc_average_profiles(void *ctx, uint64_t first_event, int n, const double *xy_proj,
                                const double *xy_targ, const double *b, int from_order, int to_order,
                                const smc_average_outputs *out, int *n_used);

/* Centrality-binned averaged profiles (the per-order mean of
 * MakeDensity::generate_profile_average, src/MakeDensity.cpp:1331-1340,
 * split into Npart classes).  Every event of [first_event, first_event + n)
 * is recentred on its density's centre of mass and rotated to its
 * order-`order` participant plane (GlueDensity::calcCMAngle,
 * src/GlueDensity.cpp:87-144), then added to its bin: bin k holds the events
 * with npart_edges[k] <= Npart1 + Npart2 < npart_edges[k + 1] (k < nbins
 * <= 64; others are left out).
 *   method 0: the sources are moved and re-splatted (MCnucl::rotateGrid,
 *             src/MCnucl.cpp:1152-1174: the reference's method, exact);
 *   method 1: each density is resampled bilinearly on the rotated frame
 *             (one splat per event; preimages beyond the grid read zero).
 * The bins are FP32 sums with compensation.  mean [nbins][nx][ny] (host)
 * receives the bin averages of rho * finalFactor (MakeDensity::setSd,
 * :2514-2522), counts [nbins] (may be NULL) the events per bin. */
smc_status smc_average_binned(void *ctx, uint64_t first_event, int n, int order, int method, int nbins,
                              const int *npart_edges, double *mean, int *counts);

/* Reverse-mode gradients of the MC-Glauber event (no reference counterpart:
 * the reference computes no derivatives).  For the events of smc_generate
 * (first_event..) or of smc_inject (xy_proj / xy_targ / b given) the
 * scalar
 *   L = sum_e  g_eps[e][0] |eps_2(e)| + g_eps[e][1] |eps_3(e)|
 *            + sum_cells g_rho[e][ix][iy] rho_e(ix, iy)
 * (eps_n with r^n weighting about the centre of mass over the hot-spot
 * region, as in columns 2-3 of the order-n block of smc_outputs.ecc;
 * rho = getRho) is differentiated with respect to
 *   grad[0] = dL/d width     (Gaussian nucleon width w, MCnucl::gaussCal)
 *   grad[1] = dL/d alpha     (WN / binary-collision mixing, MCnucl.cpp:688-779)
 *   grad[2] = dL/dR, grad[3] = dL/da  (Woods-Saxon radius and
 *            diffuseness, both nuclei together: through the nucleon
 *            positions of ws_inverse_cdf sampling, or of injected events
 *            through the given position tangents; else 0)
 * with the participants, the collisions, the splat windows, the per-cell
 * cuts, the hot-spot region and the hard-core decisions held fixed (they
 * are piecewise constant in the parameters).  The forward pass is
 * recomputed inside the call.
 * MC-Glauber (which_mc_model 5) with Gaussian entropy (shape_of_entropy 2),
 * sub_model 1 or 2.  g_eps / g_rho may be NULL (zero cotangent);
 * grad_events (may be NULL) receives the per-event gradients [n][4]. */
typedef struct smc_adjoint_args {
  int device;                /* every pointer here and the injected
                                positions are device pointers              */
  const double *g_eps;       /* [n][2]                                     */
  const float *g_rho;        /* [n][nx][ny]                                */
  const double *tangent_proj;/* injected events: [n][A][4] and [n][B][4]    */
  const double *tangent_targ;/* position tangents d(x,y)/dR, d(x,y)/da of
                                each nucleon, or NULL                      */
  double *grad_events;       /* [n][4]                                     */
} smc_adjoint_args;
smc_status smc_adjoint(void *ctx, uint64_t first_event, int n, const double *xy_proj,
                       const double *xy_targ, const double *b, const smc_adjoint_args *args,
                       double *grad);

/* Counters and kernel timing of a context (no reference counterpart; the
 * reference only times the whole run with clock(), src/main.cpp:40-68).
 * With timing enabled, CUDA events bracket every launch of the two event
 * kernels on the context's stream and their durations are summed. */
typedef struct smc_stats {
  uint64_t events;          /* events produced                              */
  uint64_t attempts;        /* sampling attempts (retries included)         */
  uint64_t launches;        /* kernels launched                             */
  uint64_t sample_launches, grid_launches;
  double sample_ms, grid_ms;/* summed kernel durations (timing enabled)     */
  uint64_t post_launches;   /* kernels after the splat: the binned
                               accumulation, the adjoint                    */
  double post_ms;
} smc_stats;
smc_status smc_set_timing(void *ctx, int enabled);
/* Splat implementation of the batched entry points (smc_generate,
 * smc_inject, smc_average); no reference counterpart (the reference has
 * one CPU loop, src/MCnucl.cpp:432-478, :688-866).  tensor_cores != 0
 * (default): the separable contraction Gx diag(w) Gy^T on the tcgen05
 * tensor cores in split-TF32 (three-term) precision with FP32
 * accumulation, plus an exact subtraction of the window cells beyond the
 * reference's cut; used for Gaussian profiles (shape_of_nucleons != 1,
 * shape_of_entropy != 1).  0: the FP32 CUDA-core splat.  The plain path
 * (smc_generate_plain) always uses the CUDA-core splat. */
smc_status smc_set_grid_path(void *ctx, int tensor_cores);
/* Launch-configuration autotuner (no reference counterpart): times the
 * context's own workload -- n_events events (0: 8192) of smc_generate with
 * device outputs, event ids from 2^62 on -- for each splat path
 * (tensor-core contraction, CUDA-core splat) and events per launch
 * (2048, 4096, 8192, 16384), keeps the fastest for the context's later calls and
 * reports the rates (events/s, tensor-core path first; 0 where a path does
 * not apply).  Both paths give the same results within FP32 rounding. */
typedef struct smc_tuning {
  int tensor_cores;         /* chosen splat path                            */
  int chunk;                /* chosen events per launch                     */
  double events_per_s[8];   /* (tensor cores, CUDA cores) x (2048 .. 16384)  */
} smc_tuning;
smc_status smc_autotune(void *ctx, int n_events, smc_tuning *out);
smc_status smc_get_stats(void *ctx, smc_stats *stats);
smc_status smc_reset_stats(void *ctx);

/* MC-KLN dN/dy table (MCnucl::makeTable, src/MCnucl.cpp:911-960): copies the
 * current table ([tmax][tmax] doubles, rapidity slice 0) to host. */
smc_status smc_kln_table(void *ctx, double *host_table, int capacity);
/* MCnucl::makeTable(ptmin, dpt, iPtmax) (src/MCnucl.cpp:967-1025): the
 * p_T-differential table dN/dy d^2p_T at p_T = pt_min + k d_pt, k < nbins
 * (the PT_Min, d_PT, MaxPT of src/MakeDensity.cpp:67-71), on the nodes
 * (i dT, j dT) of the p_T-integrated table: KLNModel::getdNdy at fixed p_T
 * (src/KLNModel.cpp:96-124, the (k_T, phi) integral of func_simpson,
 * :281-322), built on the GPU in FP64 by the k_T and phi Gauss-Legendre
 * rules of the p_T-integrated table (the reference integrates by adaptive
 * Simpson to 1e-4 relative).  The table stays in the context for
 * smc_outputs.rho_pt.  host_table (may be NULL): receives it,
 * [tmax][tmax][nbins] doubles (capacity in doubles).  MC-KLN only. */
smc_status smc_kln_pt_table(void *ctx, double pt_min, double d_pt, int nbins, double *host_table, size_t capacity);

/* Text outputs in the reference's layouts (host code, no GPU), so that the
 * reference's downstream tools read the results unchanged.
 * smc_write_ecc: MakeDensity::dumpEccentricities (src/MakeDensity.cpp:
 *   2432-2500, non-deformed layout): for each event of ecc[n][49] appends
 *   one line to the file of each order in [from_order, to_order] and one
 *   line with all orders 1..9 to the file of order 10; pattern is a printf
 *   pattern with one %d for the order ("data/sn_ecc_eccp_%d.dat").
 * smc_write_density_block: MakeDensity::dumpDensityBlock (:2597-2609):
 *   grid[nx][ny] as nx lines of ny values (%22.12g); the reference writes
 *   the entropy density getRho * finalFactor.
 * smc_write_density_4col: MakeDensity::dumpDensity4Col (:2573-2595): a
 *   header with Npart and the grid size, then rapidity, x, y, value per cell. */
smc_status smc_write_ecc(const double *ecc, int n, int from_order, int to_order, const char *pattern);
/* smc_write_ecc in the layout dumpEccentricities writes when a nucleus is
 * deformed (proj_deformed or targ_deformed = 1; src/MakeDensity.cpp:
 * 2435-2455, 2483-2492): each line of every file ends in four more fields
 * (%16.8g), cos(theta) and phi of the projectile, then of the target, from
 * orientation[n][4] (smc_outputs.orientation).  The reference prints the
 * members MCnucl::lastCx1, lastPh1, lastCx2, lastPh2 there, which its code
 * never assigns (src/MCnucl.h:90), so its files hold whatever those members
 * contain; here they hold the orientations the names describe. */
smc_status smc_write_ecc_deformed(const double *ecc, const double *orientation, int n, int from_order,
                                  int to_order, const char *pattern);
smc_status smc_write_density_block(const double *grid, int nx, int ny, const char *filename);

/* Binary counterparts of the text files (no reference counterpart: the
 * reference writes text only, src/MakeDensity.cpp:2432-2609): NumPy .npy
 * files (format 1.0, little-endian, C order; numpy.load reads them), one
 * array per text file holding the text file's columns at full precision.
 * smc_write_npy: data [shape[0]]..[shape[ndim-1]] of elem_bytes 4 (float)
 * or 8 (double), 1 <= ndim <= 4; with append != 0 an existing file this
 * function wrote with the same type and trailing dimensions grows by
 * shape[0] rows (the text writers append the same way), any other existing
 * file: SMC_ERR_ARGUMENT.  A density block is [nx][ny] (the rows of
 * sd_event_<n>_block.dat), the collision table [ncoll][2] (binary.dat).
 * smc_write_ecc_npy: sn_ecc_eccp_<order>.npy [n][9] (the per-order line's
 * Re, Im (r^2), Re, Im (r^n), <r^n>, then Npart, Ncoll, dN/dy, b) and
 * sn_ecc_eccp_10.npy [n][49]; with orientation (not NULL) the deformed
 * layout's four more columns; appends like smc_write_ecc. */
smc_status smc_write_npy(const char *filename, const void *data, int elem_bytes, int ndim, const int64_t *shape,
                         int append);
smc_status smc_write_ecc_npy(const double *ecc, const double *orientation, int n, int from_order, int to_order,
                             const char *pattern);
smc_status smc_write_density_4col(const double *grid, int nx, int ny, double xmin, double ymin, double dx, double dy,
                                  double rapidity, double npart, const char *filename);
/* MCnucl::dumpBinaryTable (src/MCnucl.cpp:1175-1189): appends one line per
 * binary collision, x and y (%10.3g each), of xy[ncoll][2]. */
smc_status smc_write_binary_table(const double *xy, int ncoll, const char *filename);
/* Nucleus::dumpParticipants / dumpNucleons (src/Nucleus.cpp:753-778) as
 * dumpBinaryTable writes them (src/MCnucl.cpp:1193-1207) for one event:
 * `participants` (wounded.data, overwritten): the wounded nucleons of the
 * projectile then the target, x, y and the nucleus id 1 or 2 (each
 * nucleus in nucleon order; the reference lists a target's participants
 * in the order they were first hit); `proj`,
 * `targ` (nucl1.data, nucl2.data, overwritten): every nucleon, x and y.
 * xy [A+B][2] and wounded [A+B] as smc_outputs.positions / .wounded; any
 * file name may be NULL. */
smc_status smc_write_nucleon_tables(const double *xy, const uint8_t *wounded, int A, int B, const char *participants,
                                    const char *proj, const char *targ);
/* MCnucl::dumpparticipantTable (src/MCnucl.cpp:1213-1220): appends the
 * event's participants (the wounded.data lines, Nucleus::dumpParticipants,
 * src/Nucleus.cpp:753-764) to `filename` (the Jet mode's
 * ParticipantTable_event_<n>.dat). */
smc_status smc_write_participant_table(const double *xy, const uint8_t *wounded, int A, int B, const char *filename);
/* MCnucl::getSpectators + dumpSpectatorsTable (src/MCnucl.cpp:1223-1265):
 * the non-participants, projectile then target in nucleon order, x, y and
 * the beam rapidity +Y (projectile) or -Y (target) of sqrt(s) = ecm
 * (scientific, 4 digits); `filename` overwritten (Spectators_event_<n>.dat). */
smc_status smc_write_spectator_table(const double *xy, const uint8_t *wounded, int A, int B, double ecm,
                                     const char *filename);
/* MakeDensity::dumpDensity5Col / dumpDesityptCol (src/MakeDensity.cpp:
 * 2612-2661): the header "% <npart>= .. xmax= .. ymax= .. Ptmax= ..", then
 * one line per cell (x-major) of its nbins p_T values times `scale`
 * (finalFactor for setSd), %22.12e each.  data [nx][ny][nbins]
 * (smc_outputs.rho_pt of one event). */
smc_status smc_write_density_pt(const float *data, int nx, int ny, int nbins, double npart, double scale,
                                const char *filename);

/* smc_inject without any device allocation.  No counterpart in the
 * reference (which allocates host arrays freely); it exists for callers that
 * may not call cudaMalloc -- a host framework that owns all device memory
 * through its own pool, or a code path that must not change the allocation
 * state (e.g. around stream capture).  The caller passes device buffers:
 * positions d_xy_proj [n][A][2], d_xy_targ [n][B][2], d_b [n] (may be NULL),
 * and the outputs d_ecc [n][49], d_rho [n][nx][ny], d_status [n] (per-event
 * smc_status).  Work is queued on cuda_stream (NULL: the legacy default
 * stream) and is complete when that stream is.
 *   - Intermediate data use one static 24 MiB device array: each event needs
 *     64 + 64 * (2 (A + B) + max_collisions) bytes (max_collisions defaults to
 *     2048 here), e.g. at most 136 Pb+Pb events per call; larger n returns
 *     SMC_ERR_SCRATCH_LIMIT.
 *   - All calls share that array: calls that overlap on the GPU (other
 *     streams, other threads) race.  Nothing in it needs clearing.
 *   - The first call on a device looks up the array's device address with
 *     that device current; make it before any stream capture.  Under lazy
 *     module loading (the CUDA default) that first call also loads the
 *     module, which commits the 24 MiB on the device: make it before the
 *     caller's pool takes the device memory, or set CUDA_MODULE_LOADING=EAGER.
 *   - max_collisions defaults to 2048 here, not smc_inject's 4096: an event
 *     with more binary collisions gets SMC_ERR_CAPACITY in d_status (set
 *     max_collisions to take such events, at fewer events per call).
 *   - MC-Glauber (which_mc_model 5) and sqrt(T_A T_B) (7) only.
 * Allocates nothing: no cudaMalloc, cudaFree or allocating library call. */
smc_status smc_inject_noalloc(const smc_params *params, int n, const double *d_xy_proj,
                              const double *d_xy_targ, const double *d_b, double *d_ecc,
                              float *d_rho, int *d_status, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
