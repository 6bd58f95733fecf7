/* FP64 CPU restatement of superMC's per-event initial-condition path.
 *
 * TEST INFRASTRUCTURE (the checker): loaded only by tests/, the smoke check
 * and bench.py's CPU-baseline / reference legs.  Compiled with
 * -ffp-contract=off so that every expression rounds exactly as the
 * reference's x86-64 build does; expressions keep the reference's operand
 * order where that changes rounding.  Citations are file:line within the
 * chunshen1987/superMC project. */
#include "smc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ================================================================== */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), own implementation */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void smco_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    if (r) { k0 += PHILOX_W0; k1 += PHILOX_W1; }
    uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double u53(uint32_t lo, uint32_t hi) {
  uint64_t v = ((uint64_t)hi << 32) | lo;
  return ((double)(v >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

/* Counter layout shared with the CUDA sampler: ctr = {slot, stream,
 * event_lo, event_hi}, key = {seed_lo, seed_hi}. */
void smco_uniform2(uint64_t seed, uint64_t event, uint32_t stream, uint32_t slot, double u[2]) {
  uint32_t ctr[4] = {slot, stream, (uint32_t)event, (uint32_t)(event >> 32)};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  smco_philox4x32(ctr, key, o);
  u[0] = u53(o[0], o[1]);
  u[1] = u53(o[2], o[3]);
}

/* stream ids (low byte of the stream word; the retry attempt is above) */
enum { ST_EVENT = 0, ST_PROJ = 1, ST_TARG = 2, ST_DEUT = 3, ST_COLL = 4, ST_FLUCT = 5, ST_NBD = 6, ST_CONF = 7 };
static uint32_t stream_id(int attempt, int sid) { return ((uint32_t)attempt << 8) | (uint32_t)sid; }

/* ================================================================== */
/* constants                                                            */

/* hadronxsec::totalXsection / elasticXsection for pp (Regge96.cpp:27-50) */
double smco_sigma_in(double ecm) {
  double s = ecm * ecm;
  double sig = 22.0 * pow(s, 0.079) + 56.1 * pow(s, -0.46);
  double bel = 2.0 * 2.3 + 2.0 * 2.3 + 4.0 * pow(s, 0.0808) - 4.2;
  double sigel = 0.0511 * sig * sig / bel;
  return sig - sigel;
}

/* Nucleus::Gauss38 (Nucleus.cpp:697-751): the 38-point Gauss-Legendre
 * rule's published abscissae/weights, mapped to [xini, xfin]. */
static void gauss38(double xini, double xfin, double *xn, double *wn) {
  static const double xp[19] = {
      4.078514790458e-2, 1.220840253379e-1, 2.025704538921e-1, 2.817088097902e-1,
      3.589724404794e-1, 4.338471694324e-1, 5.058347179279e-1, 5.744560210478e-1,
      6.392544158297e-1, 6.997986803792e-1, 7.556859037540e-1, 8.065441676053e-1,
      8.520350219324e-1, 8.918557390046e-1, 9.257413320486e-1, 9.534663309335e-1,
      9.748463285902e-1, 9.897394542664e-1, 9.980499305357e-1};
  static const double wp[19] = {
      8.152502928039e-2, 8.098249377060e-2, 7.990103324353e-2, 7.828784465821e-2,
      7.615366354845e-2, 7.351269258474e-2, 7.038250706690e-2, 6.678393797914e-2,
      6.274093339213e-2, 5.828039914700e-2, 5.343201991033e-2, 4.822806186076e-2,
      4.270315850467e-2, 3.689408159400e-2, 3.083950054518e-2, 2.457973973823e-2,
      1.815657770961e-2, 1.161344471647e-2, 5.002880749632e-3};
  double x[38], w[38];
  for (int k = 0; k < 19; k++) {
    x[19 + k] = xp[k];
    w[19 + k] = wp[k];
    x[18 - k] = -xp[k];
    w[18 - k] = wp[k];
  }
  for (int i = 0; i < 38; i++) {
    xn[i] = (xfin - xini) * x[i] / 2.0 + (xini + xfin) / 2.0;
    wn[i] = (xfin - xini) * w[i] / 2.0;
  }
}

/* GaussianNucleonsCal::getSigEff (GaussianNucleonsCal.cpp:130-163) */
double smco_sigeff(double siginNN, double width) {
  double xg[38], wg[38];
  gauss38(0.0, 1.0, xg, wg);
  double sigin = siginNN * 0.1;
  double Bmax = 5.0 * width;
  double sigeff = 10.0, sigeff0;
  int guard = 0;
  do {
    sigeff0 = sigeff;
    double sum = 0.0, dN = 0.0;
    for (int ib = 0; ib < 38; ib++) {
      double b = xg[ib] * Bmax;
      double db = wg[ib] * Bmax;
      double Tpp = exp(-b * b / (4. * width * width)) / (M_PI * (4. * width * width));
      sum += 2 * M_PI * b * db * (1.0 - exp(-sigeff * Tpp));
      dN += 2 * M_PI * b * db * Tpp * exp(-sigeff * Tpp);
    }
    sigeff -= (sum - sigin) / dN;
  } while (fabs(sigeff - sigeff0) > 1e-4 && ++guard < 1000);
  return sigeff;
}

/* HulthenFunc::CDF (HulthenFunc.cpp:27-36) */
double smco_hulthen_cdf(double r) {
  double alpha = .228;
  double beta = 1.18;
  if (r <= 0) return 0;
  const double c = (alpha * beta * (alpha + beta)) / ((alpha - beta) * (alpha - beta));
  return 2 * c *
         (2 * (exp(-r * (alpha + beta)) / (alpha + beta)) - .5 * exp(-2 * alpha * r) / alpha -
          .5 * exp(-2 * beta * r) / beta + .5 / alpha + .5 / beta - 2 / (alpha + beta));
}

/* invertFunc (arsenal.cpp:318-387) applied to the Hulthen CDF with the
 * arguments of HulthenFunc::invCDF (HulthenFunc.cpp:38-41). */
double smco_hulthen_inv(double y) {
  const double xL = 0, xR = 100.0, dx = 0.001, x0 = 1.0, rel = 0.001;
  double accuracy = dx * rel;
  double XX2 = x0, XX1 = XX2 - 10 * accuracy;
  int impatience = 0;
  while (fabs(XX2 - XX1) > accuracy) {
    XX1 = XX2;
    double F0 = smco_hulthen_cdf(XX1) - y;
    double X1 = (XX1 > xL + dx) ? XX1 - dx : xL;
    double X2 = (XX1 < xR - dx) ? XX1 + dx : xR;
    double F1 = smco_hulthen_cdf(X1), F2 = smco_hulthen_cdf(X2);
    double F3 = (F1 - F2) / (X1 - X2);
    XX2 = XX1 - F0 / F3;
    if (++impatience > 60) return NAN; /* reference: exit(-1) */
  }
  return XX2;
}

/* sixPoint2dInterp (arsenal.cpp:33-54) */
double smco_six_point(double x, double y, double v00, double v01, double v02, double v10,
                      double v11, double v20) {
  double axx = 1.0 / 2.0 * (v00 - 2 * v10 + v20);
  double axy = v00 - v01 - v10 + v11;
  double ayy = 1.0 / 2.0 * (v00 - 2 * v01 + v02);
  double bx = 1.0 / 2.0 * (-3.0 * v00 + 4 * v10 - v20);
  double by = 1.0 / 2.0 * (-3.0 * v00 + 4 * v01 - v02);
  double c = v00;
  return axx * x * x + axy * x * y + ayy * y * y + bx * x + by * y + c;
}

/* ================================================================== */
/* nucleus parameters (Nucleus.cpp:58-148)                              */
void smco_nucleus_init(smco_nucleus *n, int A, int deformed, double R_override,
                       double a_override, double dmin_override) {
  memset(n, 0, sizeof *n);
  n->A = A;
  n->deformed = deformed;
  n->d_min = 0.9; /* Nucleus.cpp:190 */
  double Ad = (double)A;
  double rad = 1.12 * pow(Ad, 0.333333) - 0.86 / pow(Ad, 0.333333);
  double dr = 0.54;
  if (A == 197) { rad = 6.42; dr = 0.45; }
  else if (A == 63) { rad = 4.28; dr = 0.5; }
  else if (A == 238) { rad = 6.86; dr = 0.44; }
  else if (A == 208) { rad = 6.67; dr = 0.44; }
  else if (A == 129) { rad = 5.36; dr = 0.590; }
  if (R_override > 0) rad = R_override;
  if (a_override > 0) dr = a_override;
  if (dmin_override > 0) n->d_min = dmin_override;
  n->R = rad;
  n->a = dr;
  if (deformed) {
    if (A == 197) { n->beta2 = -0.13; n->beta4 = -0.03; }
    else if (A == 63) { n->beta2 = 0.162; n->beta4 = 0.006; }
    else if (A == 129) { n->beta2 = 0.162; n->beta4 = -0.003; }
    else if (A == 238) { n->beta2 = 0.28; n->beta4 = 0.093; }
  }
  n->rmax_cut = rad + 2.5;
  n->rw_max = 1.0 / (1.0 + exp(-rad / dr));
}

/* Nucleus::SphericalHarmonics (Nucleus.cpp:669-694) */
static double sph_harm(int l, double ct) {
  double ylm = 0.0;
  if (l == 2) {
    ylm = 3.0 * ct * ct - 1.0;
    ylm *= 0.31539156525252005;
  } else {
    ylm = 35.0 * ct * ct * ct * ct;
    ylm -= 30.0 * ct * ct;
    ylm += 3.0;
    ylm *= 0.10578554691520431;
  }
  return ylm;
}

/* Point3D::rotate (MathBasics.cpp:41-50) */
static void rotate3(double *x, double *y, double *z, double costheta, double phi) {
  double x0 = *x, y0 = *y, z0 = *z;
  double cth = costheta, cphi = cos(phi);
  double sth = sqrt(1. - cth * cth), sphi = sin(phi);
  *x = cth * cphi * x0 - sphi * y0 + sth * cphi * z0;
  *y = cth * sphi * x0 + cphi * y0 + sth * sphi * z0;
  *z = -sth * x0 + 0. * y0 + cth * z0;
}

/* ================================================================== */
/* bounding boxes with Box2D's arithmetic (Box2D.h:49-63, Box2D.cpp:81-123) */
typedef struct { double xl, xr, yl, yr, xc, yc; } box_t;

static void box_set_center_xy(box_t *b, double x, double y) {
  b->xl += x - b->xc;
  b->xr += x - b->xc;
  b->yl += y - b->yc;
  b->yr += y - b->yc;
  b->xc = x;
  b->yc = y;
}
static void box_square(box_t *b, double size) {
  b->xl = b->xc - size / 2;
  b->xr = b->xc + size / 2;
  b->yl = b->yc - size / 2;
  b->yr = b->yc + size / 2;
}
static void box_over_union(box_t *b, const box_t *o) {
  b->xl = fmin(o->xl, b->xl);
  b->xr = fmax(o->xr, b->xr);
  b->yl = fmin(o->yl, b->yl);
  b->yr = fmax(o->yr, b->yr);
  b->xc = (b->xl + b->xr) / 2.0;
  b->yc = (b->yl + b->yr) / 2.0;
}

/* ================================================================== */
/* event state                                                          */
typedef struct {
  double x, y, z;
  box_t box, base; /* Particle::boundingBox / baseBox (Particle.h:25-26) */
  int id;          /* index before sorting: injection / acceptance order     */
  double nfx, nfy, nfz, u0; /* inverse-CDF sampling: nucleus-frame position
                               before the centre-of-mass shift and the radial
                               uniform (u0 < 0 otherwise)                   */
  int *hits;       /* who_hit_me: indices into the other nucleus, in order */
  int nhits, caphits;
} nucleon_t;

struct smco_event {
  smco_params p;
  int n[2], cap[2];
  nucleon_t *nuc[2];
  int npart[2];
  int *part[2]; /* wounded list (first-hit order), indices into nuc */
  int ncoll, capc;
  double *cx, *cy, *caw;
  int *cpa, *cpb;  /* nucleon indices (sorted arrays) of each collision */
  box_t *cbox; /* CollisionPair::boundingBox, default all zero */
  double *TA, *TB, *rho, *rhob;
  double dndy;
};

smco_event *smco_event_new(const smco_params *p) {
  smco_event *e = (smco_event *)calloc(1, sizeof *e);
  e->p = *p;
  size_t g = (size_t)p->nx * p->ny;
  e->TA = (double *)calloc(g, sizeof(double));
  e->TB = (double *)calloc(g, sizeof(double));
  e->rho = (double *)calloc(g, sizeof(double));
  e->rhob = (double *)calloc(g, sizeof(double));
  return e;
}

static void clear_nucleons(smco_event *e) {
  for (int w = 0; w < 2; w++) {
    for (int i = 0; i < e->n[w]; i++) free(e->nuc[w][i].hits);
    e->n[w] = 0;
    e->npart[w] = 0;
  }
  e->ncoll = 0;
}

void smco_event_free(smco_event *e) {
  if (!e) return;
  clear_nucleons(e);
  for (int w = 0; w < 2; w++) { free(e->nuc[w]); free(e->part[w]); }
  free(e->cx); free(e->cy); free(e->caw); free(e->cbox); free(e->cpa); free(e->cpb);
  free(e->TA); free(e->TB); free(e->rho); free(e->rhob);
  free(e);
}

static void reserve(smco_event *e, int w, int n) {
  if (n <= e->cap[w]) return;
  e->nuc[w] = (nucleon_t *)realloc(e->nuc[w], sizeof(nucleon_t) * n);
  e->part[w] = (int *)realloc(e->part[w], sizeof(int) * n);
  e->cap[w] = n;
}

/* Particle::Particle (Particle.cpp:16-24) + calculateBounds (:94-99) with
 * all quarks at the nucleon centre: base box = 8w square about the
 * construction point, bounding box = base box U the 8*quark_width quark box. */
static void construct(const smco_event *e, nucleon_t *n, double x, double y, double z) {
  n->x = x; n->y = y; n->z = z;
  box_t b = {0, 0, 0, 0, 0, 0};
  box_set_center_xy(&b, x, y);
  box_square(&b, 8 * e->p.width);
  n->base = b;
  n->box = b;
  box_t q = {0, 0, 0, 0, 0, 0};
  box_square(&q, 8 * e->p.quark_width);
  box_set_center_xy(&q, x + 0.0, y + 0.0);
  box_over_union(&n->box, &q);
  n->hits = NULL;
  n->nhits = n->caphits = 0;
  n->id = 0;
  n->nfx = n->nfy = n->nfz = 0;
  n->u0 = -1;
}

static int cmp_xleft(const void *a, const void *b);
/* records each nucleon's pre-sort index, then sorts by the box's left edge */
static void sort_nucleons(smco_event *e, int w, int n) {
  for (int i = 0; i < n; i++) e->nuc[w][i].id = i;
  qsort(e->nuc[w], n, sizeof(nucleon_t), cmp_xleft);
}

/* Particle::calculateBounds after a move (MCnucl.cpp:1161,1167): the box
 * restarts from the construction-time base box. */
static void recompute_bounds(const smco_event *e, nucleon_t *n) {
  n->box = n->base;
  box_t q = {0, 0, 0, 0, 0, 0};
  box_square(&q, 8 * e->p.quark_width);
  box_set_center_xy(&q, n->x + 0.0, n->y + 0.0);
  box_over_union(&n->box, &q);
}

static void set_x(nucleon_t *n, double a) { n->x = a; box_set_center_xy(&n->box, a, n->box.yc); }
static void set_y(nucleon_t *n, double a) { n->y = a; box_set_center_xy(&n->box, n->box.xc, a); }

static int cmp_xleft(const void *a, const void *b) {
  double xa = ((const nucleon_t *)a)->box.xl, xb = ((const nucleon_t *)b)->box.xl;
  return (xa > xb) - (xa < xb);
}

void smco_event_inject(smco_event *e, const double *xyA, int A, const double *xyB, int B) {
  clear_nucleons(e);
  const double *src[2] = {xyA, xyB};
  int cnt[2] = {A, B};
  for (int w = 0; w < 2; w++) {
    reserve(e, w, cnt[w] > 0 ? cnt[w] : 1);
    for (int i = 0; i < cnt[w]; i++) construct(e, &e->nuc[w][i], src[w][2 * i], src[w][2 * i + 1], 0.0);
    e->n[w] = cnt[w];
    sort_nucleons(e, w, cnt[w]);
  }
}

/* ================================================================== */
/* Woods-Saxon radius by inverse CDF (differentiable sampling mode; no
 * reference counterpart -- the reference samples radii by rejection,
 * Nucleus.cpp:578-621).  The density is the reference's truncated one,
 * rho(r) = 1/(1+exp((r-R)/a)) on [0, rmax], rmax = R + 2.5, with
 * N(r) = int_0^r t^2 rho dt and F = N(r)/N(rmax).  r(u) solves F(r) = u;
 * by the implicit function theorem
 *   dr/dp = -(N_p(r) - u dN(rmax)/dp) / (r^2 rho(r)),  p = R, a,
 * with N_p = int_0^r t^2 d rho/dp dt and dN(rmax)/dR including the moving
 * end point (rmax^2 rho(rmax)).  Quadrature: 8-point Gauss-Legendre on 24
 * panels (nodes and weights from the standard tables). */
static const double GL8X[4] = {0.1834346424956498, 0.5255324099163290, 0.7966664774136267, 0.9602898564975363};
static const double GL8W[4] = {0.3626837833783620, 0.3137066458778873, 0.2223810344533745, 0.1012285362903763};

static void ws_integrand(double R, double a, double t, double *f, double *fR, double *fa) {
  double rho = 1.0 / (1.0 + exp((t - R) / a));
  double d = rho * (1.0 - rho) / a;
  *f = t * t * rho;
  *fR = t * t * d;
  *fa = t * t * d * (t - R) / a;
}

static void ws_N(double R, double a, double r, double *N, double *NR, double *Na) {
  const int panels = 24;
  double h = r / panels, s = 0, sR = 0, sa = 0;
  for (int p = 0; p < panels; p++) {
    double c = (p + 0.5) * h, hh = 0.5 * h;
    for (int k = 0; k < 4; k++)
      for (int sg = -1; sg <= 1; sg += 2) {
        double f, fR, fa;
        ws_integrand(R, a, c + sg * hh * GL8X[k], &f, &fR, &fa);
        s += GL8W[k] * hh * f;
        sR += GL8W[k] * hh * fR;
        sa += GL8W[k] * hh * fa;
      }
  }
  *N = s;
  *NR = sR;
  *Na = sa;
}

double smco_ws_icdf(double R, double a, double u, double *drdR, double *drda) {
  double rmax = R + 2.5;
  double Nt, NtR, Nta;
  ws_N(R, a, rmax, &Nt, &NtR, &Nta);
  double f_end, fR_end, fa_end;
  ws_integrand(R, a, rmax, &f_end, &fR_end, &fa_end);
  NtR += f_end; /* d rmax / dR = 1 */
  double target = u * Nt, lo = 0, hi = rmax;
  for (int it = 0; it < 64; it++) {
    double mid = 0.5 * (lo + hi), N, NR, Na;
    ws_N(R, a, mid, &N, &NR, &Na);
    if (N < target) lo = mid;
    else hi = mid;
  }
  double r = 0.5 * (lo + hi);
  if (drdR || drda) {
    double N, NR, Na, f, fR, fa;
    ws_N(R, a, r, &N, &NR, &Na);
    ws_integrand(R, a, r, &f, &fR, &fa);
    double F = N / Nt;
    if (drdR) *drdR = f > 0 ? -(NR - F * NtR) / f : 0;
    if (drda) *drda = f > 0 ? -(Na - F * Nta) / f : 0;
  }
  return r;
}

/* ================================================================== */
/* sampling                                                             */

/* one Woods-Saxon candidate from four uniforms, following
 * Nucleus::getDeformRandomWS (Nucleus.cpp:578-621); returns 0 if the
 * radial (or deformed) rejection test fails. */
static int ws_candidate(const smco_nucleus *n, double ctr, double phir, const double u[4],
                        double *x, double *y, double *z) {
  double r, cx;
  if (n->deformed) {
    r = n->rmax_cut * pow(u[0], 1.0 / 3.0);
    cx = 1.0 - 2.0 * u[1];
    double y20 = sph_harm(2, cx), y40 = sph_harm(4, cx);
    double rad1 = n->R * (1.0 + n->beta2 * y20 + n->beta4 * y40);
    double rwMax1 = 1.0 / (1.0 + exp(-rad1 / n->a));
    if (u[2] * rwMax1 > 1.0 / (1.0 + exp((r - rad1) / n->a))) return 0;
    double sx = sqrt(1.0 - cx * cx);
    double phi = 2 * M_PI * u[3];
    double px = r * sx * cos(phi), py = r * sx * sin(phi), pz = r * cx;
    rotate3(&px, &py, &pz, ctr, phir);
    *x = px; *y = py; *z = pz;
  } else {
    r = n->rmax_cut * pow(u[0], 1.0 / 3.0);
    if (u[1] * n->rw_max > 1.0 / (1.0 + exp((r - n->R) / n->a))) return 0;
    cx = 1.0 - 2.0 * u[2];
    double sx = sqrt(1.0 - cx * cx);
    double phi = 2 * M_PI * u[3];
    *x = r * sx * cos(phi);
    *y = r * sx * sin(phi);
    *z = r * cx;
  }
  return 1;
}

/* Particle constructor randomness (Particle.cpp:38,50,53,54): four drand48
 * draws whose values do not move the nucleon when quarks sit at its centre */
static void particle_draws(void) {
  (void)drand48(); (void)drand48(); (void)drand48(); (void)drand48();
}

/* Nucleus::populate (Nucleus.cpp:187-317) with drand48 */
static void populate_drand48(smco_event *e, int w, const smco_nucleus *n, double xc, double yc) {
  double cx = 1.0 - 2.0 * drand48();
  double phi = 2 * M_PI * drand48();
  int A = n->A;
  reserve(e, w, A);
  e->n[w] = 0;
  if (n->conf && A >= 3) {
    /* Nucleus::GetNucleonPosition (Nucleus.cpp:555-574): configuration
     * rand() % nconf, each nucleon rotated; constructed in place
     * (:210-236) */
    const double *cfg = n->conf + (size_t)(rand() % n->nconf) * 3 * A;
    for (int i = 0; i < A; i++) {
      double x = cfg[3 * i], y = cfg[3 * i + 1], z = cfg[3 * i + 2];
      rotate3(&x, &y, &z, cx, phi);
      particle_draws();
      construct(e, &e->nuc[w][i], x + xc, y + yc, z);
    }
    e->n[w] = A;
  } else if (A == 1) {
    particle_draws();
    construct(e, &e->nuc[w][0], xc, yc, 0.0);
    e->n[w] = 1;
  } else if (A == 2) {
    double width = 1.0, dw = width * 1e-30;
    double d = smco_hulthen_inv(0 + dw + (width - 2 * dw) * drand48());
    double x1 = d / 2.0, y1 = 0, z1 = 0;
    rotate3(&x1, &y1, &z1, cx, phi);
    particle_draws();
    construct(e, &e->nuc[w][0], x1 + xc, y1 + yc, z1);
    particle_draws();
    construct(e, &e->nuc[w][1], -x1 + xc, -y1 + yc, -z1);
    e->n[w] = 2;
  } else {
    double rmin = n->d_min * n->d_min;
    double xcm = 0, ycm = 0, zcm = 0;
    for (int ia = 0; ia < A; ia++) {
      double x, y, z;
      int conflict;
      do {
        double u[4];
        int ok;
        if (n->deformed) {
          do {
            u[0] = drand48();
            u[1] = drand48();
            double r = n->rmax_cut * pow(u[0], 1.0 / 3.0);
            double ccx = 1.0 - 2.0 * u[1];
            double rad1 = n->R * (1.0 + n->beta2 * sph_harm(2, ccx) + n->beta4 * sph_harm(4, ccx));
            double rwMax1 = 1.0 / (1.0 + exp(-rad1 / n->a));
            u[2] = drand48();
            ok = !(u[2] * rwMax1 > 1.0 / (1.0 + exp((r - rad1) / n->a)));
          } while (!ok);
          u[3] = drand48();
        } else {
          do {
            u[0] = drand48();
            double r = n->rmax_cut * pow(u[0], 1.0 / 3.0);
            u[1] = drand48();
            ok = !(u[1] * n->rw_max > 1.0 / (1.0 + exp((r - n->R) / n->a)));
          } while (!ok);
          u[2] = drand48();
          u[3] = drand48();
        }
        ws_candidate(n, cx, phi, u, &x, &y, &z);
        conflict = 0;
        for (int i = 0; i < e->n[w]; i++) {
          const nucleon_t *q = &e->nuc[w][i];
          double r2 = (x - q->x) * (x - q->x) + (y - q->y) * (y - q->y) + (z - q->z) * (z - q->z);
          if (r2 < rmin) { conflict = 1; break; }
        }
      } while (conflict);
      xcm += x; ycm += y; zcm += z;
      particle_draws();
      construct(e, &e->nuc[w][e->n[w]], x, y, z);
      e->n[w]++;
    }
    for (int ia = 0; ia < A; ia++) {
      nucleon_t *q = &e->nuc[w][ia];
      double x = q->x - xcm / A + xc;
      double y = q->y - ycm / A + yc;
      double z = q->z - zcm / A;
      set_x(q, x);
      set_y(q, y);
      q->z = z;
    }
  }
  sort_nucleons(e, w, e->n[w]);
}

void smco_event_populate_drand48(smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB,
                                 double b) {
  clear_nucleons(e);
  populate_drand48(e, 0, nA, b / 2.0, 0);
  populate_drand48(e, 1, nB, -b / 2.0, 0);
}

/* The same algorithm driven by Philox streams.  Every candidate has its own
 * four uniforms (slots 2c, 2c+1 of the nucleus's stream); a rejected
 * candidate is simply skipped.  The nucleus orientation comes from the
 * event stream. Positions are built exactly as the GPU sampler builds them:
 * candidate in the nucleus frame, centre of mass removed, shifted by +-b/2.
 * As in Nucleus::populate (Nucleus.cpp:274-309) a Woods-Saxon nucleon is
 * constructed at its nucleus-frame point and then moved, so its base box
 * stays there; light nuclei are constructed in place (:199-236). */
static int populate_philox(smco_event *e, int w, const smco_nucleus *n, double xc, double yc,
                           uint64_t seed, uint64_t event, int attempt) {
  double o[2];
  smco_uniform2(seed, event, stream_id(attempt, ST_EVENT), 1 + w, o);
  double cx = 1.0 - 2.0 * o[0];
  double phi = 2 * M_PI * o[1];
  int A = n->A;
  reserve(e, w, A);
  e->n[w] = 0;
  double px[256], py[256], pz[256], pu[256];
  if (A > 256) return -1;
  int cnt = 0;
  if (n->conf && A >= 3) {
    /* configuration floor(u nconf) from the nucleus's own stream (the
     * reference: rand() % nconf), rotated in FP64, not recentred */
    double u[2];
    smco_uniform2(seed, event, stream_id(attempt, ST_CONF), (uint32_t)w, u);
    int k = (int)(u[0] * n->nconf);
    if (k > n->nconf - 1) k = n->nconf - 1;
    const double *cfg = n->conf + (size_t)k * 3 * A;
    for (int i = 0; i < A; i++) {
      px[i] = cfg[3 * i]; py[i] = cfg[3 * i + 1]; pz[i] = cfg[3 * i + 2];
      rotate3(&px[i], &py[i], &pz[i], cx, phi);
    }
    cnt = A;
  } else if (A == 1) {
    px[0] = 0; py[0] = 0; pz[0] = 0;
    cnt = 1;
  } else if (A == 2) {
    double u[2];
    smco_uniform2(seed, event, stream_id(attempt, ST_DEUT), (uint32_t)w, u);
    double d = smco_hulthen_inv(u[0]);
    double x1 = d / 2.0, y1 = 0, z1 = 0;
    rotate3(&x1, &y1, &z1, cx, phi);
    px[0] = x1; py[0] = y1; pz[0] = z1;
    px[1] = -x1; py[1] = -y1; pz[1] = -z1;
    cnt = 2;
  } else {
    double rmin = n->d_min * n->d_min;
    uint32_t sid = stream_id(attempt, w == 0 ? ST_PROJ : ST_TARG);
    for (uint32_t c = 0; cnt < A; c++) {
      if (c > 1000000u) return -2;
      double u[4];
      smco_uniform2(seed, event, sid, 2 * c, u);
      smco_uniform2(seed, event, sid, 2 * c + 1, u + 2);
      double x, y, z;
      if (n->icdf && !n->deformed) {
        /* inverse-CDF radius, the candidate's direction as in ws_candidate */
        double r = smco_ws_icdf(n->R, n->a, u[0], NULL, NULL);
        double ct = 1.0 - 2.0 * u[2], st = sqrt(1.0 - ct * ct), ph = 2 * M_PI * u[3];
        x = r * st * cos(ph);
        y = r * st * sin(ph);
        z = r * ct;
      } else if (!ws_candidate(n, cx, phi, u, &x, &y, &z)) {
        continue;
      }
      int conflict = 0;
      for (int i = 0; i < cnt; i++) {
        double r2 = (x - px[i]) * (x - px[i]) + (y - py[i]) * (y - py[i]) + (z - pz[i]) * (z - pz[i]);
        if (r2 < rmin) { conflict = 1; break; }
      }
      if (conflict) continue;
      px[cnt] = x; py[cnt] = y; pz[cnt] = z;
      pu[cnt] = (n->icdf && !n->deformed) ? u[0] : -1.0;
      cnt++;
    }
    double xcm = 0, ycm = 0, zcm = 0;
    for (int i = 0; i < cnt; i++) { xcm += px[i]; ycm += py[i]; zcm += pz[i]; }
    for (int i = 0; i < cnt; i++) {
      nucleon_t *q = &e->nuc[w][i];
      construct(e, q, px[i], py[i], pz[i]);
      q->nfx = px[i]; q->nfy = py[i]; q->nfz = pz[i]; q->u0 = pu[i];
      set_x(q, px[i] - xcm / A + xc);
      set_y(q, py[i] - ycm / A + yc);
      q->z = pz[i] - zcm / A;
    }
    e->n[w] = cnt;
    sort_nucleons(e, w, cnt);
    return 0;
  }
  for (int i = 0; i < cnt; i++) construct(e, &e->nuc[w][i], px[i] + xc, py[i] + yc, pz[i]);
  e->n[w] = cnt;
  sort_nucleons(e, w, cnt);
  return 0;
}

void smco_event_populate_philox(smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB,
                                double b, uint64_t seed, uint64_t event, int attempt) {
  clear_nucleons(e);
  populate_philox(e, 0, nA, b / 2.0, 0, seed, event, attempt);
  populate_philox(e, 1, nB, -b / 2.0, 0, seed, event, attempt);
}

/* b = sqrt((bmax^2-bmin^2) u + bmin^2) (MakeDensity.cpp:2149) */
double smco_impact_philox(uint64_t seed, uint64_t event, int attempt, double bmin, double bmax) {
  double u[2];
  smco_uniform2(seed, event, stream_id(attempt, ST_EVENT), 0, u);
  return sqrt((bmax * bmax - bmin * bmin) * u[0] + bmin * bmin);
}

/* ================================================================== */
/* pairing                                                              */
static void add_hit(nucleon_t *n, int other) {
  if (n->nhits == n->caphits) {
    n->caphits = n->caphits ? 2 * n->caphits : 8;
    n->hits = (int *)realloc(n->hits, sizeof(int) * n->caphits);
  }
  n->hits[n->nhits++] = other;
}

/* MCnucl::hit (MCnucl.cpp:357-385) for criteria 1 and 2 */
static int hit(const smco_event *e, const nucleon_t *p1, const nucleon_t *p2, double u) {
  double b = sqrt((p2->x - p1->x) * (p2->x - p1->x) + (p2->y - p1->y) * (p2->y - p1->y));
  int crit = e->p.collision_criterion;
  if (crit != 1 && crit != 2) crit = e->p.shape_of_entropy == 2 ? 2 : 1;
  if (crit == 1) return (b * b <= e->p.dsq) ? 1 : 0;
  double w = e->p.width;
  return u < 1. - exp(-e->p.sigma_gg * exp(-b * b / (4. * w * w)) / (4. * M_PI * w * w));
}

/* stream for the criterion-2 test of pair (i,j): set by the caller */
static uint64_t g_pair_seed, g_pair_event;
static int g_pair_attempt, g_pair_philox;

/* Gamma(k, theta) from the Philox stream of one source: the method of
 * Marsaglia and Tsang ("A simple method for generating gamma variables",
 * ACM TOMS 26 (2000) 363), with Gamma(k) = Gamma(k+1) U^(1/k) for k < 1 and
 * Box-Muller normals.  Iteration t draws counters 32 slot + 2t, 2t + 1
 * (t < 15), the k < 1 uniform counter 32 slot + 31.  The reference draws
 * the same distribution from GSL (gsl_ran_gamma, MCnucl.cpp:1285,1298). */
static double gamma_stream(uint64_t seed, uint64_t event, uint32_t sid, uint32_t base, double k, double theta);
double smco_gamma_philox(uint64_t seed, uint64_t event, int attempt, uint32_t slot, double k, double theta) {
  return gamma_stream(seed, event, stream_id(attempt, ST_FLUCT), 32 * slot, k, theta);
}

/* Gamma(k, theta) from counters base + 2t, base + 2t + 1 and base + 31 */
static double gamma_stream(uint64_t seed, uint64_t event, uint32_t sid, uint32_t base, double k, double theta) {
  double kk = k < 1 ? k + 1 : k;
  double d = kk - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  double g = d; /* after 15 rejections (probability below 1e-19) */
  for (int t = 0; t < 15; t++) {
    double u[2], w[2];
    smco_uniform2(seed, event, sid, base + 2 * t, u);
    smco_uniform2(seed, event, sid, base + 2 * t + 1, w);
    double x = sqrt(-2.0 * log(1.0 - u[0])) * cos(2.0 * M_PI * u[1]);
    double v = 1.0 + c * x;
    if (v <= 0) continue;
    v = v * v * v;
    if (log(1.0 - w[0]) < 0.5 * x * x + d - d * v + d * log(v)) {
      g = d * v;
      break;
    }
  }
  if (k < 1) {
    double u[2];
    smco_uniform2(seed, event, sid, base + 31, u);
    g *= pow(1.0 - u[0], 1.0 / k);
  }
  return g * theta;
}

void smco_set_pair_stream(uint64_t seed, uint64_t event, int attempt, int philox) {
  g_pair_seed = seed;
  g_pair_event = event;
  g_pair_attempt = attempt;
  g_pair_philox = philox;
}

int smco_event_pair(smco_event *e) {
  nucleon_t *P = e->nuc[0], *T = e->nuc[1];
  int nP = e->n[0], nT = e->n[1];
  e->npart[0] = e->npart[1] = 0;
  int start = 0;
  for (int ip = 0; ip < nP; ip++) {
    box_t pb = P[ip].box, tb = {0, 0, 0, 0, 0, 0};
    while (start < nT) {
      tb = T[start].box;
      if (tb.xr >= pb.xl) break;
      start++;
    }
    int i = start;
    while (i < nT && pb.xr >= tb.xl) {
      tb = T[i].box;
      if (pb.yl <= tb.yr && pb.yr >= tb.yl) {
        double u = 0;
        int crit = e->p.collision_criterion;
        if (crit != 1 && crit != 2) crit = e->p.shape_of_entropy == 2 ? 2 : 1;
        if (crit == 2) {
          if (g_pair_philox) {
            double uu[2];
            smco_uniform2(g_pair_seed, g_pair_event, stream_id(g_pair_attempt, ST_COLL),
                          (uint32_t)(ip * nT + i), uu);
            u = uu[0];
          } else {
            u = drand48();
          }
        }
        if (hit(e, &P[ip], &T[i], u)) {
          add_hit(&P[ip], i);
          add_hit(&T[i], ip);
          if (P[ip].nhits == 1) e->part[0][e->npart[0]++] = ip;
          if (T[i].nhits == 1) e->part[1][e->npart[1]++] = i;
        }
      }
      i++;
    }
  }
  /* MCnucl::createBinaryCollisions (MCnucl.cpp:326-352) */
  int nc = 0;
  for (int k = 0; k < e->npart[0]; k++) nc += P[e->part[0][k]].nhits;
  if (nc > e->capc) {
    e->capc = nc;
    e->cx = (double *)realloc(e->cx, sizeof(double) * nc);
    e->cy = (double *)realloc(e->cy, sizeof(double) * nc);
    e->caw = (double *)realloc(e->caw, sizeof(double) * nc);
    e->cbox = (box_t *)realloc(e->cbox, sizeof(box_t) * nc);
    e->cpa = (int *)realloc(e->cpa, sizeof(int) * nc);
    e->cpb = (int *)realloc(e->cpb, sizeof(int) * nc);
  }
  e->ncoll = 0;
  for (int k = 0; k < e->npart[0]; k++) {
    const nucleon_t *p = &P[e->part[0][k]];
    for (int j = 0; j < p->nhits; j++) {
      const nucleon_t *t = &T[p->hits[j]];
      int c = e->ncoll++;
      e->cpa[c] = e->part[0][k];
      e->cpb[c] = p->hits[j];
      e->cx[c] = (p->x + t->x) / 2.0;
      e->cy[c] = (p->y + t->y) / 2.0;
      double aw = 0.;
      if (e->p.which_mc_model == 5 && e->p.sub_model == 2) {
        aw += 1 / p->nhits; /* integer division, as in the reference */
        aw += 1 / t->nhits;
      }
      e->caw[c] = aw;
      memset(&e->cbox[c], 0, sizeof(box_t));
    }
  }
  return e->ncoll;
}

int smco_event_npart(const smco_event *e, int which) { return e->npart[which]; }
int smco_event_ncoll(const smco_event *e) { return e->ncoll; }

int smco_event_nucleons(const smco_event *e, int which, double *xyz, int maxn) {
  for (int i = 0; i < e->n[which] && i < maxn; i++) {
    xyz[3 * i] = e->nuc[which][i].x;
    xyz[3 * i + 1] = e->nuc[which][i].y;
    xyz[3 * i + 2] = e->nuc[which][i].z;
  }
  return e->n[which];
}
int smco_event_participants(const smco_event *e, int which, double *xy, int maxn) {
  for (int i = 0; i < e->npart[which] && i < maxn; i++) {
    const nucleon_t *q = &e->nuc[which][e->part[which][i]];
    xy[2 * i] = q->x;
    xy[2 * i + 1] = q->y;
  }
  return e->npart[which];
}
int smco_event_participant_index(const smco_event *e, int which, int *idx, int maxn) {
  for (int i = 0; i < e->npart[which] && i < maxn; i++) idx[i] = e->part[which][i];
  return e->npart[which];
}
int smco_event_collisions(const smco_event *e, double *xy, int maxn) {
  for (int i = 0; i < e->ncoll && i < maxn; i++) {
    xy[2 * i] = e->cx[i];
    xy[2 * i + 1] = e->cy[i];
  }
  return e->ncoll;
}

/* ================================================================== */
/* grids                                                                */
#define G(a, i, j) (a)[(size_t)(i) * e->p.ny + (j)]

/* Particle::getSmoothTn (Particle.cpp:122-132) */
static double smooth_tn(double width, double px, double py, double xg, double yg) {
  double r = sqrt((xg - px) * (xg - px) + (yg - py) * (yg - py));
  if (r > 5 * width) return 0;
  return (1 / (2 * M_PI * width * width)) * exp(-r * r / (2 * width * width));
}

static void window(const smco_event *e, double lo, double hi, double mn, double d, int nmax,
                   int *a, int *b) {
  int l = (int)((lo - mn) / d);
  int r = (int)((hi - mn) / d);
  *a = l > 0 ? l : 0;
  *b = r < nmax ? r : nmax;
  (void)e;
}

/* MCnucl::setThickness (MCnucl.cpp:432-478) */
static void set_thickness(smco_event *e, int w, double *TA) {
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  double d_max = e->p.shape_of_nucleons == 1 ? 2. * sqrt(e->p.dsq) : 5. * e->p.width;
  for (int k = 0; k < e->npart[w]; k++) {
    const nucleon_t *q = &e->nuc[w][e->part[w][k]];
    double x = q->x, y = q->y;
    int xl, xr, yl, yr;
    window(e, x - d_max, x + d_max, Xmin, dx, e->p.nx, &xl, &xr);
    window(e, y - d_max, y + d_max, Ymin, dy, e->p.ny, &yl, &yr);
    for (int ix = xl; ix < xr; ix++) {
      double xg = Xmin + ix * dx;
      for (int iy = yl; iy < yr; iy++) {
        double yg = Ymin + iy * dy;
        double dc = (x - xg) * (x - xg) + (y - yg) * (y - yg);
        if (e->p.shape_of_nucleons == 1) {
          if (dc > e->p.dsq) continue;
          G(TA, ix, iy) += 10.0 / e->p.sigin;
        } else {
          G(TA, ix, iy) += smooth_tn(e->p.width, x, y, xg, yg);
        }
      }
    }
  }
}

int smco_event_thickness(smco_event *e) {
  size_t g = (size_t)e->p.nx * e->p.ny;
  memset(e->TA, 0, g * sizeof(double));
  memset(e->TB, 0, g * sizeof(double));
  set_thickness(e, 0, e->TA);
  set_thickness(e, 1, e->TB);
  if (e->p.which_mc_model == 1) {
    int imax = 0;
    for (size_t k = 0; k < g; k++) {
      int i = (int)((e->TA[k]) / (10.0 / e->p.sigin) + 0.5);
      int j = (int)((e->TB[k]) / (10.0 / e->p.sigin) + 0.5);
      if (i > imax) imax = i;
      if (j > imax) imax = j;
    }
    /* MCnucl.cpp:424-428; MCnucl::makeTable has already replaced tmax by
     * its subdivided value when events run */
    if (imax >= e->p.kln_tmax) return 2;
  }
  return 0;
}

/* MCnucl::sampleFluctuationFactorforParticipant / ...forBinaryCollision
 * (MCnucl.cpp:1271-1301), cc_fluctuation_model 6: mean-one Gamma weights,
 * k = (1 - alpha + eps)/(2 theta) per participant and (alpha + eps)/theta
 * per binary collision.  Slots: participant i (sorted order) of nucleus w
 * is w A + i; collision (i, j) is A + B + i B + j. */
static double part_fluct(const smco_event *e, int w, int i) {
  if (e->p.cc_fluctuation_model != 6) return 1.0;
  const double eps = 1e-8, th = e->p.cc_fluctuation_gamma_theta;
  const double k = (1 - e->p.alpha + eps) / 2. / th, theta = 2. / (1 - e->p.alpha + eps) * th;
  return smco_gamma_philox(g_pair_seed, g_pair_event, g_pair_attempt, (uint32_t)(w ? e->n[0] + i : i), k, theta);
}
static double coll_fluct(const smco_event *e, int c) {
  if (e->p.cc_fluctuation_model != 6) return 1.0;
  const double eps = 1e-8, th = e->p.cc_fluctuation_gamma_theta;
  const double k = (e->p.alpha + eps) / th, theta = th / (e->p.alpha + eps);
  uint32_t slot = (uint32_t)(e->n[0] + e->n[1] + e->cpa[c] * e->n[1] + e->cpb[c]);
  return smco_gamma_philox(g_pair_seed, g_pair_event, g_pair_attempt, slot, k, theta);
}

/* MCnucl::addDensity (MCnucl.cpp:822-866), shape_of_entropy 1 and 2 */
static void add_density(smco_event *e, int w, double *dens) {
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  for (int k = 0; k < e->npart[w]; k++) {
    const nucleon_t *q = &e->nuc[w][e->part[w][k]];
    const double f = part_fluct(e, w, e->part[w][k]);   /* Particle::getSmoothDensity's fluctfactor */
    double x = q->x, y = q->y;
    int xl = (int)((q->box.xl - Xmin) / dx), xr = (int)((q->box.xr - Xmin) / dx);
    int yl = (int)((q->box.yl - Ymin) / dy), yr = (int)((q->box.yr - Ymin) / dy);
    if (xl < 0) xl = 0;
    if (xr > e->p.nx) xr = e->p.nx;
    if (yl < 0) yl = 0;
    if (yr > e->p.ny) yr = e->p.ny;
    for (int ir = xl; ir < xr; ir++) {
      double xg = Xmin + ir * dx;
      for (int jr = yl; jr < yr; jr++) {
        double yg = Ymin + jr * dy;
        double dc = (x - xg) * (x - xg) + (y - yg) * (y - yg);
        if (e->p.shape_of_entropy == 1) {
          if (dc > e->p.dsq) continue;
          G(dens, ir, jr) += 10.0 / e->p.sigin * f;
        } else {
          G(dens, ir, jr) += smooth_tn(e->p.width, x, y, xg, yg) * f;
        }
      }
    }
  }
}

/* pow(double, int) as the reference's C++98 build evaluates it: the
 * integer-exponent overload of <cmath> (binary exponentiation, right to
 * left), not libm pow.  Used wherever the reference passes an int exponent
 * (GlueDensity.cpp:126, MakeDensity.cpp:2291,2410-2418). */
static double powi(double x, int m) {
  unsigned int n = m < 0 ? -(unsigned int)m : (unsigned int)m;
  double y = (n % 2) ? x : 1;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1 / y : y;
}

static double peak_height(double w) { return 1 / (2 * M_PI * w * w); }


/* Poisson(lambda) from counters base.. (inversion below 10, else the
 * transformed rejection of Hoermann, Insurance: Mathematics and Economics
 * 12 (1993) 39) */
static double poisson_stream(uint64_t seed, uint64_t event, uint32_t sid, uint32_t base, double lam) {
  if (!(lam > 0)) return 0;
  if (lam < 10) {
    double u[2];
    smco_uniform2(seed, event, sid, base, u);
    double p = exp(-lam), s = p;
    int n = 0;
    while (u[0] > s && n < 1000) {
      n++;
      p *= lam / n;
      s += p;
    }
    return n;
  }
  double slam = sqrt(lam), loglam = log(lam);
  double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
  double invalpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2);
  for (int t = 0; t < 32; t++) {
    double uv[2];
    smco_uniform2(seed, event, sid, base + t, uv);
    double U = uv[0] - 0.5, V = uv[1];
    double us = 0.5 - fabs(U);
    double kf = floor((2 * a / us + b) * U + lam + 0.43);
    if (us >= 0.07 && V <= vr) return kf;
    if (kf < 0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + kf * loglam - lgamma(kf + 1)) return kf;
  }
  return floor(lam + 0.5);
}

/* MCnucl::fluctuateCurrentDensity (MCnucl.cpp:869-905): every cell's density
 * becomes n/(dx dy), n negative-binomial with mean nb = rho dx dy and shape
 * k (constant, model 1; kpp min(T_A, T_B) sigma/10, model 2), drawn as
 * Poisson(Gamma(k, nb/k)) from the cell's Philox stream (the event's stream
 * set by smco_set_pair_stream; counters 64 cell + ...) */
static void fluctuate_density(smco_event *e) {
  const int model = e->p.cc_fluctuation_model;
  const double area = e->p.dx * e->p.dy;
  const double kpp = 1.0 / M_PI * area * 1.0 * (0.25 * 0.25 / 0.197327053 / 0.197327053);
  const uint32_t sid = stream_id(0, ST_NBD);
  size_t g = (size_t)e->p.nx * e->p.ny;
  for (size_t c = 0; c < g; c++) {
    double nb = e->rho[c] * area, k = e->p.cc_fluctuation_k;
    if (model == 2) {
      k = kpp * fmin(e->TA[c], e->TB[c]) * e->p.sigin / 10;
      if (nb < 1e-10) continue;
    }
    if (!(nb > 0) || !(k > 0)) { e->rho[c] = 0; continue; }
    double lam = gamma_stream(g_pair_seed, g_pair_event, sid, (uint32_t)(64 * c), k, nb / k);
    e->rho[c] = poisson_stream(g_pair_seed, g_pair_event, sid, (uint32_t)(64 * c + 32), lam) / area;
  }
}

double smco_nbd_draw(uint64_t seed, uint64_t event, uint32_t cell, double nb, double k) {
  const uint32_t sid = stream_id(0, ST_NBD);
  double lam = gamma_stream(seed, event, sid, 64 * cell, k, nb / k);
  return poisson_stream(seed, event, sid, 64 * cell + 32, lam);
}

int smco_event_density(smco_event *e) {
  size_t g = (size_t)e->p.nx * e->p.ny;
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  double w = e->p.width, w2 = w * w;
  double dc_sq_max = 25. * w2;
  double d_max = e->p.shape_of_nucleons == 1 ? 2. * sqrt(e->p.dsq) : 5. * w;
  double alpha = e->p.alpha;
  e->dndy = 0.0;
  if (e->p.which_mc_model == 1) {
    /* MCnucl.cpp:654-687 */
    if (!e->p.kln_table) return 5;
    int tmax = e->p.kln_tmax;
    const double *T = e->p.kln_table;
    for (int ir = 0; ir < e->p.nx; ir++)
      for (int jr = 0; jr < e->p.ny; jr++) {
        double di = G(e->TA, ir, jr) / e->p.kln_dT;
        double dj = G(e->TB, ir, jr) / e->p.kln_dT;
        if ((di < 0 || di >= tmax - 2) || (dj < 0 || dj >= tmax - 2)) return 4;
        int i = (int)floor(di), j = (int)floor(dj);
        double v = smco_six_point(di - i, dj - j, T[(size_t)i * tmax + j], T[(size_t)i * tmax + j + 1],
                                  T[(size_t)i * tmax + j + 2], T[(size_t)(i + 1) * tmax + j],
                                  T[(size_t)(i + 1) * tmax + j + 1], T[(size_t)(i + 2) * tmax + j]);
        G(e->rho, ir, jr) = v;
        e->dndy += v;
      }
  } else if (e->p.which_mc_model == 5) {
    /* MCnucl.cpp:688-779 */
    double *rhop = (double *)calloc(g, sizeof(double));
    double *tab = (double *)calloc(g, sizeof(double));
    if (e->p.sub_model == 1) {
      add_density(e, 0, rhop);
      add_density(e, 1, rhop);
      double prefactor = (1.0 - alpha) / 2.;
      for (size_t k = 0; k < g; k++) rhop[k] = rhop[k] * prefactor;
    } else if (e->p.sub_model != 2) {
      free(rhop); free(tab);
      return 5;
    }
    if (alpha > 1e-8) {
      for (int c = 0; c < e->ncoll; c++) {
        double x = e->cx[c], y = e->cy[c];
        double fw = alpha + (1. - alpha) * e->caw[c];
        double f = coll_fluct(e, c);   /* CollisionPair::getfluctfactor, MCnucl.cpp:730-731 */
        int xl, xr, yl, yr;
        window(e, x - d_max, x + d_max, Xmin, dx, e->p.nx, &xl, &xr);
        window(e, y - d_max, y + d_max, Ymin, dy, e->p.ny, &yl, &yr);
        for (int ir = xl; ir < xr; ir++) {
          double xg = Xmin + ir * dx;
          for (int jr = yl; jr < yr; jr++) {
            double yg = Ymin + jr * dy;
            double dc = (x - xg) * (x - xg) + (y - yg) * (y - yg);
            if (e->p.shape_of_entropy == 1) {
              if (dc <= e->p.dsq) tab[(size_t)ir * e->p.ny + jr] += f * (10.0 / e->p.sigin) * fw;
            } else {
              if (dc <= dc_sq_max)
                tab[(size_t)ir * e->p.ny + jr] +=
                    f * peak_height(w) * exp(-dc / (2 * w2)) * fw;
            }
          }
        }
      }
    }
    for (size_t k = 0; k < g; k++) {
      double d = rhop[k] + tab[k];
      e->rho[k] = d;
      e->dndy += d;
    }
    free(rhop); free(tab);
  } else if (e->p.which_mc_model == 7) {
    /* MCnucl.cpp:780-811 */
    double *ra = (double *)calloc(g, sizeof(double));
    double *rb = (double *)calloc(g, sizeof(double));
    add_density(e, 0, ra);
    add_density(e, 1, rb);
    for (size_t k = 0; k < g; k++) {
      double d = sqrt(ra[k] * rb[k]);
      e->rho[k] = d;
      e->dndy += d;
    }
    free(ra); free(rb);
  } else {
    return 5;
  }
  if (e->dndy < 1e-15) return 3;
  if (e->p.cc_fluctuation_model == 1 || e->p.cc_fluctuation_model == 2) fluctuate_density(e);
  return 0;
}

/* The MC-Glauber density (Gaussian entropy) of the event with its structure
 * held fixed: the participant and collision windows, the per-cell cuts
 * (r <= 5 w0, dc <= 25 w0^2) and the boxes are those of the event as built
 * (width w0 = e->p.width, the nucleon positions of the event); the
 * Gaussians, the peak height 1/(2 pi w^2) and the mixing weights take
 * (w, alpha), and each Gaussian is centred on its source displaced by
 * dA / dB ([A][2], [B][2] by nucleon id, NULL = none; a collision moves by
 * the mean of its two nucleons' displacements).  With no displacement, at
 * w = w0 and alpha = e->p.alpha, this is smco_event_density.  The function
 * the adjoint's gradients are checked against by finite differences. */
int smco_event_density_moved(smco_event *e, double w, double alpha, const double *dA, const double *dB,
                             double *rho) {
  size_t g = (size_t)e->p.nx * e->p.ny;
  if (e->p.which_mc_model != 5 || e->p.shape_of_entropy == 1) return 5;
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  double w0 = e->p.width;
  double d_max = e->p.shape_of_nucleons == 1 ? 2. * sqrt(e->p.dsq) : 5. * w0;
  const double *disp[2] = {dA, dB};
  memset(rho, 0, sizeof(double) * g);
  if (e->p.sub_model == 1) {
    double pre = (1.0 - alpha) / 2.;
    for (int nw = 0; nw < 2; nw++)
      for (int k = 0; k < e->npart[nw]; k++) {
        const nucleon_t *q = &e->nuc[nw][e->part[nw][k]];
        const double f = part_fluct(e, nw, e->part[nw][k]);
        double x = q->x, y = q->y;
        double mx = x, my = y;
        if (disp[nw]) { mx += disp[nw][2 * q->id]; my += disp[nw][2 * q->id + 1]; }
        int xl = (int)((q->box.xl - Xmin) / dx), xr = (int)((q->box.xr - Xmin) / dx);
        int yl = (int)((q->box.yl - Ymin) / dy), yr = (int)((q->box.yr - Ymin) / dy);
        if (xl < 0) xl = 0;
        if (xr > e->p.nx) xr = e->p.nx;
        if (yl < 0) yl = 0;
        if (yr > e->p.ny) yr = e->p.ny;
        for (int ir = xl; ir < xr; ir++)
          for (int jr = yl; jr < yr; jr++) {
            double xg = Xmin + ir * dx, yg = Ymin + jr * dy;
            double r = sqrt((xg - x) * (xg - x) + (yg - y) * (yg - y));
            if (r > 5 * w0) continue;
            double r2 = (xg - mx) * (xg - mx) + (yg - my) * (yg - my);
            G(rho, ir, jr) += f * pre * peak_height(w) * exp(-r2 / (2 * w * w));
          }
      }
  } else if (e->p.sub_model != 2) {
    return 5;
  }
  for (int c = 0; c < e->ncoll; c++) {
    double x = e->cx[c], y = e->cy[c];
    double mx = x, my = y;
    const nucleon_t *pa = &e->nuc[0][e->cpa[c]], *pb = &e->nuc[1][e->cpb[c]];
    if (dA) { mx += 0.5 * dA[2 * pa->id]; my += 0.5 * dA[2 * pa->id + 1]; }
    if (dB) { mx += 0.5 * dB[2 * pb->id]; my += 0.5 * dB[2 * pb->id + 1]; }
    double fw = alpha + (1. - alpha) * e->caw[c];
    double f = coll_fluct(e, c);
    int xl, xr, yl, yr;
    window(e, x - d_max, x + d_max, Xmin, dx, e->p.nx, &xl, &xr);
    window(e, y - d_max, y + d_max, Ymin, dy, e->p.ny, &yl, &yr);
    for (int ir = xl; ir < xr; ir++)
      for (int jr = yl; jr < yr; jr++) {
        double xg = Xmin + ir * dx, yg = Ymin + jr * dy;
        double dc = (x - xg) * (x - xg) + (y - yg) * (y - yg);
        if (dc > 25. * w0 * w0) continue;
        double dm = (mx - xg) * (mx - xg) + (my - yg) * (my - yg);
        G(rho, ir, jr) += f * peak_height(w) * exp(-dm / (2 * w * w)) * fw;
      }
  }
  return 0;
}

int smco_event_density_frozen(smco_event *e, double w, double alpha, double *rho) {
  return smco_event_density_moved(e, w, alpha, NULL, NULL, rho);
}

/* Inverse-CDF-sampled nuclei: the lab-frame displacement of every nucleon
 * (by id) when (R, a) of both nuclei change by (dR, da) with the radial
 * uniforms and directions held, the centre-of-mass shift included
 * (positions = nucleus-frame points minus their mean, Nucleus.cpp:293-309);
 * and the tangents d(x, y)/dR, d(x, y)/da ([n][4] by id). */
static void icdf_moves(const smco_event *e, int w, const smco_nucleus *nu, double dR, double da, double *d,
                       double *tan) {
  int n = e->n[w];
  double m[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; i++) {
    const nucleon_t *q = &e->nuc[w][i];
    double v[4] = {0, 0, 0, 0};
    if (q->u0 >= 0) {
      double drdR, drda;
      double r0 = smco_ws_icdf(nu->R, nu->a, q->u0, &drdR, &drda);
      double s = 0;
      if (d) s = smco_ws_icdf(nu->R + dR, nu->a + da, q->u0, NULL, NULL) / r0 - 1.0;
      v[0] = d ? q->nfx * s : q->nfx * drdR / r0;
      v[1] = d ? q->nfy * s : q->nfy * drdR / r0;
      v[2] = q->nfx * drda / r0;
      v[3] = q->nfy * drda / r0;
    }
    for (int c = 0; c < 4; c++) m[c] += v[c];
    if (d) { d[2 * q->id] = v[0]; d[2 * q->id + 1] = v[1]; }
    if (tan) for (int c = 0; c < 4; c++) tan[4 * q->id + c] = v[c];
  }
  for (int i = 0; i < n; i++) {
    int id = e->nuc[w][i].id;
    if (d) { d[2 * id] -= m[0] / n; d[2 * id + 1] -= m[1] / n; }
    if (tan) for (int c = 0; c < 4; c++) tan[4 * id + c] -= m[c] / n;
  }
}

void smco_event_icdf_displacement(const smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB, double dR,
                                  double da, double *dA, double *dB) {
  icdf_moves(e, 0, nA, dR, da, dA, NULL);
  icdf_moves(e, 1, nB, dR, da, dB, NULL);
}

void smco_event_icdf_tangents(const smco_event *e, const smco_nucleus *nA, const smco_nucleus *nB, double *tA,
                              double *tB) {
  icdf_moves(e, 0, nA, 0, 0, NULL, tA);
  icdf_moves(e, 1, nB, 0, 0, NULL, tB);
}

int smco_event_nucleon_ids(const smco_event *e, int which, int *ids, int maxn) {
  int n = e->n[which] < maxn ? e->n[which] : maxn;
  for (int i = 0; i < n; i++) ids[i] = e->nuc[which][i].id;
  return n;
}

/* MCnucl::calculate_rho_binary (MCnucl.cpp:481-531), Gaussian shapes */
void smco_event_rho_binary(smco_event *e) {
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  double w = e->p.width, w2 = w * w;
  double d_max = e->p.shape_of_nucleons == 1 ? 2. * sqrt(e->p.dsq) : 5. * w;
  memset(e->rhob, 0, sizeof(double) * e->p.nx * e->p.ny);
  for (int c = 0; c < e->ncoll; c++) {
    double x = e->cx[c], y = e->cy[c];
    int xl, xr, yl, yr;
    window(e, x - d_max, x + d_max, Xmin, dx, e->p.nx, &xl, &xr);
    window(e, y - d_max, y + d_max, Ymin, dy, e->p.ny, &yl, &yr);
    for (int ir = xl; ir < xr; ir++) {
      double xg = Xmin + ir * dx;
      for (int jr = yl; jr < yr; jr++) {
        double yg = Ymin + jr * dy;
        double dc = (x - xg) * (x - xg) + (y - yg) * (y - yg);
        if (e->p.shape_of_nucleons == 1) {
          if (dc <= e->p.dsq) G(e->rhob, ir, jr) += (10.0 / e->p.sigin);
        } else {
          if (dc > 25. * w2) continue;
          G(e->rhob, ir, jr) += peak_height(w) * exp(-dc / (2 * w2));
        }
      }
    }
  }
}

void smco_event_grid(const smco_event *e, int which, double *out) {
  const double *src = which == 0 ? e->TA : which == 1 ? e->TB : which == 2 ? e->rho : e->rhob;
  memcpy(out, src, sizeof(double) * e->p.nx * e->p.ny);
}

/* The hot-spot region of dumpEccentricities: MCnucl::getHotSpots
 * (MCnucl.cpp:1303-1323) -- participant boxes of both nuclei, then the
 * collision boxes -- marked on the lattice of their union
 * (MakeDensity.cpp:2341-2359).  Returns the [nX][nY] flags (caller frees)
 * and the lattice's offset on the grid. */
static unsigned char *hotspot_region(const smco_event *e, int *nX, int *nY, int *ioff_out, int *joff_out) {
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  int nh = e->npart[0] + e->npart[1] + e->ncoll;
  box_t *hs = (box_t *)malloc(sizeof(box_t) * (nh > 0 ? nh : 1));
  int k = 0;
  for (int w = 0; w < 2; w++)
    for (int i = 0; i < e->npart[w]; i++) hs[k++] = e->nuc[w][e->part[w][i]].box;
  for (int c = 0; c < e->ncoll; c++) hs[k++] = e->cbox[c];
  box_t region = hs[0];
  for (int i = 1; i < nh; i++) box_over_union(&region, &hs[i]);
  int nYpoints = (int)((region.yr - region.yl) / dy);
  int nXpoints = (int)((region.xr - region.xl) / dx);
  unsigned char *imp = (unsigned char *)calloc((size_t)(nXpoints > 0 ? nXpoints : 1) *
                                                   (nYpoints > 0 ? nYpoints : 1), 1);
  for (int i = 0; i < nh; i++) {
    int x0 = (int)((hs[i].xl - region.xl) / dx), x1 = (int)((hs[i].xr - region.xl) / dx);
    int y0 = (int)((hs[i].yl - region.yl) / dy), y1 = (int)((hs[i].yr - region.yl) / dx);
    for (int xi = x0; xi < x1; xi++)
      for (int yi = y0; yi < y1; yi++)
        if (xi >= 0 && xi < nXpoints && yi >= 0 && yi < nYpoints)
          imp[(size_t)xi * nYpoints + yi] = 1;
  }
  *nX = nXpoints;
  *nY = nYpoints;
  *ioff_out = (int)((region.xl - Xmin) / dx);
  *joff_out = (int)((region.yl - Ymin) / dy);
  free(hs);
  return imp;
}

void smco_event_hotspot_mask(const smco_event *e, unsigned char *mask) {
  int nX, nY, ioff, joff;
  unsigned char *imp = hotspot_region(e, &nX, &nY, &ioff, &joff);
  memset(mask, 0, (size_t)e->p.nx * e->p.ny);
  for (int iR = 0; iR < nX; iR++)
    for (int jR = 0; jR < nY; jR++) {
      int i = iR + ioff, j = jR + joff;
      if (imp[(size_t)iR * nY + jR] && i >= 0 && i < e->p.nx && j >= 0 && j < e->p.ny)
        mask[(size_t)i * e->p.ny + j] = 1;
    }
  free(imp);
}

/* ================================================================== */
/* eccentricities (MakeDensity.cpp:2244-2511)                           */
void smco_event_eccentricities(smco_event *e, int from_order, int to_order, double b,
                               double *out) {
  const int max_order = 10;
  const double eps = 1e-15;
  int nx = e->p.nx, ny = e->p.ny;
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  double ff = e->p.final_factor;
  size_t g = (size_t)nx * ny;
  double *dens = (double *)malloc(sizeof(double) * g);
  for (size_t k = 0; k < g; k++) dens[k] = e->rho[k] * ff; /* MakeDensity::setSd :2514-2522 */
  double mom_real[10] = {0}, mom_imag[10] = {0}, norm[10] = {0};
  double momp_real[10] = {0}, momp_imag[10] = {0}, normp[10] = {0};
  double rn[10] = {0};
  double xc = 0, yc = 0, total = 0, density_norm = 0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double x = Xmin + i * dx, y = Ymin + j * dy;
      xc += x * dens[(size_t)i * ny + j];
      yc += y * dens[(size_t)i * ny + j];
      total += dens[(size_t)i * ny + j];
    }
  xc /= total;
  yc /= total;
  for (int ix = 0; ix < nx; ix++) {
    double x_o = Xmin + ix * dx - xc;
    for (int j = 0; j < ny; j++) {
      double y_o = Ymin + j * dy - yc;
      double r_o = sqrt(x_o * x_o + y_o * y_o);
      for (int io = 0; io < max_order; io++) rn[io] += powi(r_o, io) * dens[(size_t)ix * ny + j];
      density_norm += dens[(size_t)ix * ny + j];
    }
  }
  for (int io = 0; io < max_order; io++) rn[io] /= density_norm;

  int nXpoints, nYpoints, ioff, joff;
  unsigned char *imp = hotspot_region(e, &nXpoints, &nYpoints, &ioff, &joff);
  for (int order = from_order; order <= to_order; order++) {
    for (int iR = 0; iR < nXpoints; iR++)
      for (int jR = 0; jR < nYpoints; jR++) {
        if (!imp[(size_t)iR * nYpoints + jR]) continue;
        int i = iR + ioff, j = jR + joff;
        double x = Xmin + i * dx - xc, y = Ymin + j * dy - yc;
        double r = sqrt(x * x + y * y), theta = atan2(y, x);
        if (i < nx && i >= 0 && j < ny && j >= 0) {
          double d = dens[(size_t)i * ny + j];
          mom_real[order] += r * r * cos(order * theta) * d;
          mom_imag[order] += r * r * sin(order * theta) * d;
          norm[order] += r * r * d;
          if (order == 1) {
            momp_real[order] += powi(r, 3) * cos(order * theta) * d;
            momp_imag[order] += powi(r, 3) * sin(order * theta) * d;
            normp[order] += powi(r, 3) * d;
          } else {
            momp_real[order] += powi(r, order) * cos(order * theta) * d;
            momp_imag[order] += powi(r, order) * sin(order * theta) * d;
            normp[order] += powi(r, order) * d;
          }
        }
      }
    mom_real[order] = -mom_real[order] / (norm[order] + eps);
    mom_imag[order] = -mom_imag[order] / (norm[order] + eps);
    momp_real[order] = -momp_real[order] / (normp[order] + eps);
    momp_imag[order] = -momp_imag[order] / (normp[order] + eps);
  }
  for (int order = 1; order < max_order; order++) {
    double *o = out + 5 * (order - 1);
    o[0] = mom_real[order];
    o[1] = mom_imag[order];
    o[2] = momp_real[order];
    o[3] = momp_imag[order];
    o[4] = rn[order];
  }
  out[45] = e->npart[0] + e->npart[1];
  out[46] = e->ncoll;
  out[47] = total * dx * dy;
  out[48] = b;
  free(imp);
  free(dens);
}

/* GlueDensity::calcCMAngle (GlueDensity.cpp:87-144) */
void smco_event_cm_angle(const smco_event *e, int n, double *xcm, double *ycm, double *angle) {
  int nx = e->p.nx, ny = e->p.ny;
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  double weight = 0, X = 0, Y = 0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double x = Xmin + i * dx, y = Ymin + j * dy;
      double wei = e->rho[(size_t)i * ny + j] * dx * dy;
      weight += wei;
      X += x * wei;
      Y += y * wei;
    }
  X /= weight;
  Y /= weight;
  double nr = 0, ni = 0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double x = Xmin + i * dx - X, y = Ymin + j * dy - Y;
      double th = atan2(y, x);
      double wei = e->rho[(size_t)i * ny + j];
      double rwei = powi(sqrt(x * x + y * y), n);
      nr += rwei * cos(n * th) * wei;
      ni += rwei * sin(n * th) * wei;
    }
  *xcm = X;
  *ycm = Y;
  *angle = -atan2(-ni, -nr) / n;
}

/* The spectators (nucleons without a collision, MCnucl::getSpectators,
 * MCnucl.cpp:1223-1248) follow recenterGrid's shift (:1145-1149) and, with
 * rotate, rotateGrid's rotation (:1172-1173; a Spectator's z is never set,
 * and the rotation about z does not mix it into x, y). */
static void move_spectators(smco_event *e, double X, double Y, int rotate, double ang) {
  for (int w = 0; w < 2; w++)
    for (int i = 0; i < e->n[w]; i++) {
      nucleon_t *q = &e->nuc[w][i];
      if (q->nhits) continue;
      q->x = q->x - X;
      q->y = q->y - Y;
      if (rotate) {
        double z = 0;
        rotate3(&q->x, &q->y, &z, cos(0.0), ang);
      }
    }
}

/* MCnucl::calculate_spectator_density (MCnucl.cpp:534-614): projectile
 * spectators into A, target spectators into B */
void smco_event_spectator_density(const smco_event *e, double *A, double *B) {
  double Xmin = -e->p.xmax, Ymin = -e->p.ymax, dx = e->p.dx, dy = e->p.dy;
  double w = e->p.width, w2 = w * w;
  double d_max = e->p.shape_of_nucleons == 1 ? 2. * sqrt(e->p.dsq) : 5. * w;
  memset(A, 0, sizeof(double) * e->p.nx * e->p.ny);
  memset(B, 0, sizeof(double) * e->p.nx * e->p.ny);
  for (int nw = 0; nw < 2; nw++)
    for (int i = 0; i < e->n[nw]; i++) {
      const nucleon_t *q = &e->nuc[nw][i];
      if (q->nhits) continue;
      double *out = nw == 0 ? A : B;
      double x = q->x, y = q->y;
      int xl, xr, yl, yr;
      window(e, x - d_max, x + d_max, Xmin, dx, e->p.nx, &xl, &xr);
      window(e, y - d_max, y + d_max, Ymin, dy, e->p.ny, &yl, &yr);
      for (int ir = xl; ir < xr; ir++) {
        double xg = Xmin + ir * dx;
        for (int jr = yl; jr < yr; jr++) {
          double yg = Ymin + jr * dy;
          double dc = (x - xg) * (x - xg) + (y - yg) * (y - yg);
          if (e->p.shape_of_nucleons == 1) {
            if (dc <= e->p.dsq) G(out, ir, jr) += (10.0 / e->p.sigin);
          } else {
            if (dc > 25. * w2) continue;
            G(out, ir, jr) += peak_height(w) * exp(-dc / (2 * w2));
          }
        }
      }
    }
}

/* MCnucl::recenterGrid (MCnucl.cpp:1119-1150): shifts every source by the
 * density's centre of mass (the boxes move with Box2D::setCenter), then
 * calculateThickness and setDensity -- the reaction-plane-frame step of
 * MakeDensity.cpp:1291-1293 */
int smco_event_recenter_resplat(smco_event *e, int order) {
  double X, Y, ang;
  smco_event_cm_angle(e, order, &X, &Y, &ang);
  for (int w = 0; w < 2; w++)
    for (int k = 0; k < e->npart[w]; k++) {
      nucleon_t *q = &e->nuc[w][e->part[w][k]];
      set_x(q, q->x - X);
      set_y(q, q->y - Y);
    }
  for (int c = 0; c < e->ncoll; c++) {
    e->cx[c] = e->cx[c] - X;
    box_set_center_xy(&e->cbox[c], e->cx[c], e->cbox[c].yc);
    e->cy[c] = e->cy[c] - Y;
    box_set_center_xy(&e->cbox[c], e->cbox[c].xc, e->cy[c]);
  }
  move_spectators(e, X, Y, 0, 0.0);
  int rc = smco_event_thickness(e);
  if (rc) return rc;
  return smco_event_density(e);
}

/* MCnucl::recenterGrid + rotateGrid (MCnucl.cpp:1119-1174), then
 * calculateThickness and setDensity (MakeDensity.cpp:1331-1333) */
int smco_event_rotate_resplat(smco_event *e, int order) {
  double X, Y, ang;
  smco_event_cm_angle(e, order, &X, &Y, &ang);
  for (int w = 0; w < 2; w++)
    for (int k = 0; k < e->npart[w]; k++) {
      nucleon_t *q = &e->nuc[w][e->part[w][k]];
      set_x(q, q->x - X);
      set_y(q, q->y - Y);
    }
  for (int c = 0; c < e->ncoll; c++) {
    e->cx[c] = e->cx[c] - X;
    box_set_center_xy(&e->cbox[c], e->cx[c], e->cbox[c].yc);
    e->cy[c] = e->cy[c] - Y;
    box_set_center_xy(&e->cbox[c], e->cbox[c].xc, e->cy[c]);
  }
  for (int w = 0; w < 2; w++)
    for (int k = 0; k < e->npart[w]; k++) {
      nucleon_t *q = &e->nuc[w][e->part[w][k]];
      rotate3(&q->x, &q->y, &q->z, cos(0.0), ang);
      box_set_center_xy(&q->box, q->x, q->box.yc);
      box_set_center_xy(&q->box, q->box.xc, q->y);
      recompute_bounds(e, q);
    }
  for (int c = 0; c < e->ncoll; c++) {
    double z = 0;
    rotate3(&e->cx[c], &e->cy[c], &z, cos(0.0), ang);
  }
  move_spectators(e, X, Y, 1, ang);
  int rc = smco_event_thickness(e);
  if (rc) return rc;
  return smco_event_density(e);
}

/* ================================================================== */
/* MC-KLN (KLNModel.cpp, KLNfunc.h, KLNModel.h)                         */
static const double KLN_HBARC = 0.197327053;

void smco_kln_init(smco_kln *k, double ecm, double lambda) {
  k->ecm = ecm;
  k->lambda = lambda;
  k->y = 0.0;
  k->ptmin = 0.1;
  k->ptmax = 12.0;
  k->lambda_qcd = 0.2;
  k->alpha_max = 0.5;
  k->g2hfac = 2. * 1.0;
}

static double kln_alpha(const smco_kln *k, double q2) {
  double l2 = k->lambda_qcd * k->lambda_qcd;
  double beta0 = (33.0 - 2.0 * 3.0) / (12 * M_PI);
  if (q2 <= l2) return k->alpha_max;
  double v = 1.0 / (beta0 * log(q2 / l2));
  return k->alpha_max < v ? k->alpha_max : v;
}

static double kln_wave(const smco_kln *k, double qs2, double x, double kt2) {
  double CF = (3.0 * 3.0 - 1.0) / (2 * 3.0);
  double fac = CF * 2. / (3. * M_PI * M_PI);
  double rapdep = pow(1.0 - x, 4.);
  double alp = kln_alpha(k, qs2);
  double f = (kt2 <= qs2) ? fac / alp : fac * qs2 / kt2 / alp;
  return f * rapdep;
}

double smco_kln_integrand(const smco_kln *k, double ta, double tb, const double xv[3]) {
  double Ptmin = k->ptmin, Ptmax = k->ptmax;
  double pt = Ptmin + xv[0] * (Ptmax - Ptmin);
  double ktmax = pt;
  double kt = ktmax * xv[1];
  double phi = 2 * M_PI * xv[2];
  double ktsq1 = 0.25 * (pt * pt + kt * kt + 2 * kt * pt * cos(phi));
  double ktsq2 = 0.25 * (pt * pt + kt * kt - 2 * pt * kt * cos(phi));
  double mt = pt;
  double x1 = mt / k->ecm * exp(k->y);
  double x2 = mt / k->ecm / exp(k->y);
  if (x1 > 1.0 || x2 > 1.0) return 0.0;
  double qs2a = ta * 2. / 1.53 * pow(0.01 / x1, k->lambda);
  double qs2b = tb * 2. / 1.53 * pow(0.01 / x2, k->lambda);
  double fnc = kln_wave(k, qs2a, x1, ktsq1) * kln_wave(k, qs2b, x2, ktsq2);
  double scale = ktsq1 > ktsq2 ? ktsq1 : ktsq2;
  double alp = kln_alpha(k, scale > mt * mt ? scale : mt * mt);
  double result = alp * fnc;
  result *= 2.0 * M_PI * (Ptmax - Ptmin) * pt;
  result /= mt * mt;
  result *= 2.0 * M_PI * kt * ktmax;
  result /= 4.0;
  result *= 1.0;
  return result;
}

/* Gauss-Legendre rule on [0,1]: roots of P_n by Newton's method from the
 * Chebyshev-like initial guess cos(pi (i+3/4)/(n+1/2)), weights
 * 2/((1-x^2) P_n'(x)^2), then mapped to [0,1]. */
void smco_gauss_legendre01(int n, double *xo, double *wo) {
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
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
      if (fabs(z - z1) < 1e-15) break;
    }
    double w = 2.0 / ((1.0 - z * z) * dp * dp);
    xo[i] = 0.5 * (1.0 - z);
    xo[n - 1 - i] = 0.5 * (1.0 + z);
    wo[i] = wo[n - 1 - i] = 0.5 * w;
  }
}

double smco_kln_dndy(const smco_kln *k, double ta, double tb, int npt, int nkt, int nphi) {
  double *xp = (double *)malloc(sizeof(double) * 2 * (npt + nkt + nphi));
  double *wp = xp + npt, *xk = wp + npt, *wk = xk + nkt, *xf = wk + nkt, *wf = xf + nphi;
  smco_gauss_legendre01(npt, xp, wp);
  smco_gauss_legendre01(nkt, xk, wk);
  smco_gauss_legendre01(nphi, xf, wf);
  double sum = 0;
  for (int a = 0; a < npt; a++) {
    double sa = 0;
    for (int b = 0; b < nkt; b++) {
      double sb = 0;
      for (int c = 0; c < nphi; c++) {
        double x[3] = {xp[a], xk[b], xf[c]};
        sb += wf[c] * smco_kln_integrand(k, ta, tb, x);
      }
      sa += wk[b] * sb;
    }
    sum += wp[a] * sa;
  }
  free(xp);
  double CF = (3.0 * 3.0 - 1.0) / (2 * 3.0);
  double Norm = 2. / CF / (KLN_HBARC * KLN_HBARC);
  return 1.0 * k->g2hfac * Norm * sum * 9. / 32.;
}

/* KLNModel::getdNdy at a fixed p_T (src/KLNModel.cpp:96-124, the pt > 0
 * branch): g2hfac Norm 9/32 times the integral of func_simpson (:281-322)
 * over k_T in [0, pt] and phi in [0, 2 pi] -- alpha_s(max(k1^2, k2^2,
 * m_T^2)) phi_A(k1^2) phi_B(k2^2) k_T / m_T^2 / 4 with m_T = p_T --
 * taken by the Gauss-Legendre rules of nkt and nphi nodes (the reference
 * integrates by adaptive Simpson, relative precision 1e-4: SimpsonPrecision,
 * :27).  The rows of MCnucl::makeTable(ptmin, dpt, iPtmax),
 * src/MCnucl.cpp:967-1025. */
double smco_kln_dndy_pt(const smco_kln *k, double ta, double tb, double pt, int nkt, int nphi) {
  double *xk = (double *)malloc(sizeof(double) * 2 * (nkt + nphi));
  double *wk = xk + nkt, *xf = wk + nkt, *wf = xf + nphi;
  smco_gauss_legendre01(nkt, xk, wk);
  smco_gauss_legendre01(nphi, xf, wf);
  double mt = pt;
  double x1 = mt / k->ecm * exp(k->y), x2 = mt / k->ecm / exp(k->y);
  double sum = 0;
  if (!(x1 > 1.0 || x2 > 1.0) && pt > 0) {
    double qs2a = ta * 2. / 1.53 * pow(0.01 / x1, k->lambda);
    double qs2b = tb * 2. / 1.53 * pow(0.01 / x2, k->lambda);
    for (int b = 0; b < nkt; b++) {
      double kt = pt * xk[b], sb = 0;
      for (int c = 0; c < nphi; c++) {
        double phi = 2 * M_PI * xf[c];
        double ktsq1 = 0.25 * (pt * pt + kt * kt + 2 * kt * pt * cos(phi));
        double ktsq2 = 0.25 * (pt * pt + kt * kt - 2 * pt * kt * cos(phi));
        double fnc = kln_wave(k, qs2a, x1, ktsq1) * kln_wave(k, qs2b, x2, ktsq2);
        double scale = ktsq1 > ktsq2 ? ktsq1 : ktsq2;
        double alp = kln_alpha(k, scale > mt * mt ? scale : mt * mt);
        double result = alp * fnc;
        result *= kt;
        result /= mt * mt;
        result /= 4.0;
        sb += wf[c] * (2 * M_PI) * result;
      }
      sum += wk[b] * pt * sb;
    }
  }
  free(xk);
  double CF = (3.0 * 3.0 - 1.0) / (2 * 3.0);
  double Norm = 2. / CF / (KLN_HBARC * KLN_HBARC);
  return 1.0 * k->g2hfac * Norm * sum * 9. / 32.;
}

/* ================================================================== */
/* op-9 event loop (MakeDensity.cpp:2108-2240) for CPU-baseline timing  */
long smco_run_ecc_table(const smco_params *p, const smco_nucleus *nA, const smco_nucleus *nB,
                        double bmin, double bmax, int nev, int from_order, int to_order,
                        long seed, int use_philox, uint64_t first_event, double *out) {
  smco_event *e = smco_event_new(p);
  long tries = 0;
  if (!use_philox) srand48(seed);
  for (int ev = 0; ev < nev; ev++) {
    double b = 0;
    int attempt = 0;
    for (;;) {
      tries++;
      if (use_philox) {
        b = smco_impact_philox((uint64_t)seed, first_event + ev, attempt, bmin, bmax);
        g_pair_philox = 1;
        g_pair_seed = (uint64_t)seed;
        g_pair_event = first_event + ev;
        g_pair_attempt = attempt;
        smco_event_populate_philox(e, nA, nB, b, (uint64_t)seed, first_event + ev, attempt);
      } else {
        b = sqrt((bmax * bmax - bmin * bmin) * drand48() + bmin * bmin);
        g_pair_philox = 0;
        smco_event_populate_drand48(e, nA, nB, b);
      }
      int nc = smco_event_pair(e);
      int np = e->npart[0] + e->npart[1];
      attempt++;
      if (nc > 0 && np >= p->npmin && np <= p->npmax) break;
      if (attempt > 100000) { smco_event_free(e); return -1; }
    }
    if (smco_event_thickness(e)) { smco_event_free(e); return -2; }
    if (smco_event_density(e)) { smco_event_free(e); return -3; }
    smco_event_eccentricities(e, from_order, to_order, b, out + (size_t)49 * ev);
  }
  g_pair_philox = 0;
  smco_event_free(e);
  return tries;
}
