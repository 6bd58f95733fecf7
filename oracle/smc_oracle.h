/* FP64 CPU restatement of superMC's per-event initial-condition path.
 *
 * TEST INFRASTRUCTURE: this is the checker.  Only tests/, the smoke check and
 * the CPU-baseline leg of bench.py load it; the product path never does.
 * Each function cites the reference file:line it restates (paths are within
 * the chunshen1987/superMC project).  Its parity is pinned against the
 * reference compiled from source (oracle/Makefile.ref, oracle/ref_harness.cpp)
 * by tests/test_oracle_vs_reference.py and by the committed fixtures in
 * tests/golden/. */
#ifndef SMC_ORACLE_H
#define SMC_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* counter-based random numbers (Philox4x32-10, Salmon et al. SC'11)   */
void smco_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* two uniforms in (0,1) with 53 random bits each from one Philox block */
void smco_uniform2(uint64_t seed, uint64_t event, uint32_t stream, uint32_t slot, double u[2]);

/* ------------------------------------------------------------------ */
/* constants                                                            */
double smco_sigma_in(double ecm);                      /* Regge96.cpp:27-50     */
double smco_sigeff(double sigin_mb, double width);     /* GaussianNucleonsCal.cpp:130-163 */
double smco_hulthen_cdf(double r);                     /* HulthenFunc.cpp:27-36 */
double smco_hulthen_inv(double u);                     /* HulthenFunc.cpp:38-41 + arsenal.cpp:318-387 */
double smco_six_point(double x, double y, double v00, double v01, double v02, double v10,
                      double v11, double v20);        /* arsenal.cpp:33-54     */

/* ------------------------------------------------------------------ */
/* nucleus description (Nucleus.cpp:22-170) with optional overrides     */
typedef struct {
  int A;                /* mass number; 1 = proton, 2 = deuteron (Hulthen)  */
  int deformed;         /* 0/1                                              */
  double R, a;          /* Woods-Saxon radius and diffuseness [fm]          */
  double beta2, beta4;  /* deformation                                      */
  double d_min;         /* hard-core distance [fm] (reference: 0.9)         */
  double rmax_cut;      /* proposal sphere radius, R + 2.5                  */
  double rw_max;        /* 1/(1+exp(-R/a))                                  */
  int icdf;             /* 1: radii by inverse CDF (spherical A > 2)        */
  /* light-nucleus configurations [nconf][A][3] (NULL: Woods-Saxon); an
   * event takes one, rotated and shifted, not recentred
   * (Nucleus.cpp:210-236, 555-574) */
  const double *conf;
  int nconf;
} smco_nucleus;
/* inverse-CDF Woods-Saxon radius for the uniform u, with dr/dR, dr/da
 * (either may be NULL) */
double smco_ws_icdf(double R, double a, double u, double *drdR, double *drda);
/* Fills the reference's hard-coded parameters for mass number A; any of
 * R, a, d_min that is > 0 on input of the *_override arguments replaces
 * the reference value (reference behaviour when all are <= 0). */
void smco_nucleus_init(smco_nucleus *n, int A, int deformed, double R_override,
                       double a_override, double dmin_override);

/* ------------------------------------------------------------------ */
/* event state                                                          */
typedef struct {
  int nx, ny;               /* Maxx, Maxy                           */
  double xmax, ymax, dx, dy;
  double width;             /* gaussCal->width                      */
  double quark_width;       /* Quark::width (parameter quark_width) */
  double dsq;               /* 0.1*sigma_in/pi (MCnucl.cpp:120)     */
  double sigin;             /* sigma_in [mb]                        */
  double sigma_gg;          /* GaussianNucleonsCal sigma_gg [fm^2]  */
  double alpha;
  int which_mc_model, sub_model;
  int shape_of_nucleons, shape_of_entropy, collision_criterion;
  double final_factor;
  int npmin, npmax;
  /* KLN lookup table (row-major tmax x tmax), MCnucl.cpp:911-960 */
  const double *kln_table;
  int kln_tmax;
  double kln_dT;
  /* multiplicity fluctuations: 6 = Gamma-distributed weight per participant
   * and binary collision (MCnucl.cpp:1271-1301), drawn from the Philox
   * streams set by smco_set_pair_stream; 0 = none */
  int cc_fluctuation_model;
  double cc_fluctuation_gamma_theta;
  double cc_fluctuation_k;   /* NBD shape of model 1 */
} smco_params;
/* negative-binomial count (mean nb, shape k) of one cell's stream, as
 * fluctuateCurrentDensity draws it */
double smco_nbd_draw(uint64_t seed, uint64_t event, uint32_t cell, double nb, double k);
/* Gamma(k, theta) variate of one source (slot) of an event's fluctuation
 * stream */
double smco_gamma_philox(uint64_t seed, uint64_t event, int attempt, uint32_t slot, double k, double theta);

typedef struct smco_event smco_event;
smco_event *smco_event_new(const smco_params *p);
void smco_event_free(smco_event *e);

/* nucleons constructed directly at (x,y) (the injection harness's
 * construction: boxes are centred on the given positions), sorted by the
 * left edge of their bounding box like Nucleus::populate (Nucleus.cpp:314) */
void smco_event_inject(smco_event *e, const double *xyA, int A, const double *xyB, int B);
/* reference sampler, consuming libc drand48 in the reference's order
 * (Nucleus.cpp:187-317, 578-621; Particle.cpp:32-54) */
void smco_event_populate_drand48(smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB,
                                 double b);
/* Philox sampler used by the GPU path: same algorithm, uniforms from
 * smco_uniform2(seed, event, stream, slot).  attempt selects the retry. */
void smco_event_populate_philox(smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB,
                                double b, uint64_t seed, uint64_t event, int attempt);
double smco_impact_philox(uint64_t seed, uint64_t event, int attempt, double bmin, double bmax);

/* random draws of the Gaussian collision criterion: libc drand48 in the
 * reference's sweep order (philox = 0) or Philox streams keyed by the sorted
 * pair index (philox = 1, the GPU's streams) */
void smco_set_pair_stream(uint64_t seed, uint64_t event, int attempt, int philox);
/* MCnucl::getBinaryCollision (MCnucl.cpp:217-308); returns Ncoll */
int smco_event_pair(smco_event *e);
int smco_event_npart(const smco_event *e, int which);
int smco_event_ncoll(const smco_event *e);
/* nucleons (x,y,z) in sorted order; returns count */
int smco_event_nucleons(const smco_event *e, int which, double *xyz, int maxn);
/* participants (x,y) in first-hit order; returns count */
int smco_event_participants(const smco_event *e, int which, double *xy, int maxn);
/* participant indices into the sorted nucleon list, first-hit order */
int smco_event_participant_index(const smco_event *e, int which, int *idx, int maxn);
int smco_event_collisions(const smco_event *e, double *xy, int maxn);

/* MCnucl::calculateThickness (MCnucl.cpp:398-430); returns 0 or an error
 * code (2 = KLN table overflow, MCnucl.cpp:424-428) */
int smco_event_thickness(smco_event *e);
/* MCnucl::setDensity(0,-1) (MCnucl.cpp:626-820); 0 or error code
 * (3 = zero dN/dy, 4 = KLN lookup out of table, 5 = bad model) */
int smco_event_density(smco_event *e);
/* 0 = T_A, 1 = T_B, 2 = rho, 3 = rho_binary (MCnucl.cpp:481-531) */
void smco_event_grid(const smco_event *e, int which, double *out);
void smco_event_rho_binary(smco_event *e);
/* MakeDensity::dumpEccentricities (MakeDensity.cpp:2244-2511) on
 * rho*final_factor.  out[49]: for orders 1..9 (Re,Im r^2-weighted, Re,Im
 * r^n-weighted, <r^n>), then Npart, Ncoll, integral*dx*dy, b. */
void smco_event_eccentricities(smco_event *e, int from_order, int to_order, double b,
                               double *out);
/* the hot-spot region of the eccentricities as [nx][ny] flags */
void smco_event_hotspot_mask(const smco_event *e, unsigned char *mask);
/* model-5 density with windows, cuts and boxes of the event's own width and
 * the Gaussians and weights of (w, alpha); 0 or 5 (unsupported model) */
int smco_event_density_frozen(smco_event *e, double w, double alpha, double *rho);
/* the same with the Gaussians centred on sources displaced by dA [A][2],
 * dB [B][2] (by nucleon id, NULL = none) */
int smco_event_density_moved(smco_event *e, double w, double alpha, const double *dA, const double *dB,
                             double *rho);
/* inverse-CDF events: nucleon displacements [n][2] for (R, a) += (dR, da)
 * and tangents [n][4] = (dx/dR, dy/dR, dx/da, dy/da), by nucleon id */
void smco_event_icdf_displacement(const smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB, double dR,
                                  double da, double *dA, double *dB);
void smco_event_icdf_tangents(const smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB, double *tA,
                              double *tB);
/* pre-sort index (injection / acceptance order) of each nucleon in sorted order */
int smco_event_nucleon_ids(const smco_event *e, int which, int *ids, int maxn);
/* MCnucl::calculate_spectator_density (MCnucl.cpp:534-614) into A, B [nx][ny] */
void smco_event_spectator_density(const smco_event *e, double *A, double *B);
/* GlueDensity::calcCMAngle (GlueDensity.cpp:87-144) on rho */
void smco_event_cm_angle(const smco_event *e, int n, double *xcm, double *ycm, double *angle);
/* MCnucl::rotateGrid (MCnucl.cpp:1152-1174) + calculateThickness +
 * setDensity, i.e. one averaged-mode step (MakeDensity.cpp:1331-1333) */
int smco_event_rotate_resplat(smco_event *e, int order);
/* MCnucl::recenterGrid (MCnucl.cpp:1119-1150) + calculateThickness +
 * setDensity: the reaction-plane-frame step (MakeDensity.cpp:1291-1293) */
int smco_event_recenter_resplat(smco_event *e, int order);

/* ------------------------------------------------------------------ */
/* MC-KLN                                                               */
typedef struct {
  double ecm, lambda, y;    /* sqrt(s) [GeV], saturation exponent, rapidity */
  double ptmin, ptmax;      /* 0.1, 12 GeV (KLNModel.cpp:70-71)            */
  double lambda_qcd;        /* 0.2 GeV                                      */
  double alpha_max;         /* 0.5                                          */
  double g2hfac;            /* 2 x normalization                            */
} smco_kln;
void smco_kln_init(smco_kln *k, double ecm, double lambda);
/* KLNModel::func at the unit-cube point x[3] (KLNModel.cpp:219-277) */
double smco_kln_integrand(const smco_kln *k, double ta, double tb, const double x[3]);
/* Gauss-Legendre nodes/weights on [0,1] (own Golub-Welsch-free Newton) */
void smco_gauss_legendre01(int n, double *x, double *w);
/* dN/dy(T_A,T_B) by the deterministic tensor-product rule
 * (npt x nkt x nphi on the unit cube), times g2hfac*Norm*9/32
 * (KLNModel.cpp:97-125) */
double smco_kln_dndy(const smco_kln *k, double ta, double tb, int npt, int nkt, int nphi);
double smco_kln_dndy_pt(const smco_kln *k, double ta, double tb, double pt, int nkt, int nphi);

/* ------------------------------------------------------------------ */
/* whole event loop (MakeDensity::generateEccTable, MakeDensity.cpp:2108)
 * for CPU-baseline timing.  Uses drand48 seeded with seed when
 * use_philox == 0, else the Philox streams.  Writes nev rows of 49
 * doubles (smco_event_eccentricities layout).  Returns total tries. */
long smco_run_ecc_table(const smco_params *p, const smco_nucleus *nA, const smco_nucleus *nB,
                        double bmin, double bmax, int nev, int from_order, int to_order,
                        long seed, int use_philox, uint64_t first_event, double *out);

#ifdef __cplusplus
}
#endif
#endif
