// Device-side definitions shared by the sm_103a kernels of supermc_gb300.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace smc {

constexpr int kMaxA = 256;          // nucleons per nucleus held on chip
constexpr int kEccLen = 49;         // dumpEccentricities line length
constexpr int kMaxOrder = 10;

// Source kinds of the splat (which window rule and weight apply).
enum SrcKind : int {
  SRC_PART_BOX = 0,   // participant, bounding-box window, r <= 5w cut (MCnucl::addDensity)
  SRC_COLL = 1,       // binary collision, +-d_max window, dc <= 25 w^2 (MCnucl::setDensity)
  SRC_THICK = 2,      // participant, +-d_max window, r <= 5w (MCnucl::setThickness)
  // 3: a participant's record for the eccentricity mask only (no splat)
  SRC_SPECT = 4,      // spectator (non-participant), +-d_max window; splatted only
                      // through the averaged mode's spectator view (MCnucl::getSpectators)
  SRC_BINARY = 5,     // binary collision kept only for the averaged mode's rho_binary
                      // view (no density source: MC-KLN, alpha = 0); kinds >= 3 are
                      // never splatted directly
  SRC_RAW_BASE = 32,  // flag: participant box built at (bx, by), then moved
  SRC_AW_SHIFT = 6,   // bits 6-7: a binary collision's additional weight (sub_model 2)
};

// One source of the density/thickness splat.  Windows are grid index
// half-open ranges computed exactly as the reference's (int) casts.
struct Source {
  double x, y;        // FP64 position
  int16_t xl, xr, yl, yr;  // splat window [xl,xr) x [yl,yr)
  int16_t mx0, mx1, my0, my1;  // eccentricity-mask window (participant boxes)
  int16_t kind, plane;   // SrcKind, accumulator plane
  float weight;          // multiplies exp(-r^2/2w^2)
  float bx, by;          // construction point of a participant box (kind bit SRC_RAW_BASE)
  // the position in grid units, split into a cell (exact in FP32) and the
  // fraction within it: x = xmin + (gi0 + gfx) dx, y = ymin + (gj0 + gfy) dy
  // (set_grid_offsets; the splats' Gaussian arguments are taken from them)
  float gi0, gfx, gj0, gfy;
};
static_assert(sizeof(Source) == 64, "Source layout");

// Averaged-mode state of one source: construction position and the
// current bounding box with Box2D's centre (src/Box2D.h:16-63).
struct AvgSrc {
  double x0, y0;
  double bxl, bxr, byl, byr, bxc, byc;
};

struct NucleusDev {
  int A, deformed;
  double R, a, beta2, beta4, d_min, rmax_cut, rw_max;
  // FP32 roundings of the above (set by the sampler): R, a, rmax_cut, rw_max,
  // beta2, beta4 and d_min^2 (rounded after the FP64 square); the sampler's
  // z slabs (count, inverse thickness) of the hard-core search
  float R_f, a_f, rmax_f, rw_max_f, beta2_f, beta4_f, dmin2_f;
  int nslab;
  float slab_inv_w;
  // inverse-CDF radii (NULL table: rejection sampling).  icdf holds the
  // cumulative integrals N, dN/dR, dN/da of r^2 rho(r) at r_k = k icdf_h,
  // k < icdf_m (three rows of icdf_m); icdf_ntot = N(rmax) and its
  // derivatives, the moving end point rmax = R + 2.5 included.
  // A fourth row of icdf_nb + 1 entries holds, for u = b / icdf_nb, the
  // largest node k with N[k] <= u N(rmax) (where the search starts).
  const double *icdf;
  int icdf_m, icdf_nb;
  double icdf_h, icdf_ntot, icdf_dntot_R, icdf_dntot_a;
  // configuration table of a light nucleus ([nconf][A][3] nucleus-frame
  // positions, fm; NULL: Woods-Saxon sampling).  Each event takes one
  // configuration, rotates it by the nucleus orientation and shifts it,
  // without recentring (Nucleus::populate and GetNucleonPosition,
  // src/Nucleus.cpp:210-236, 555-574)
  const double *conf;
  int nconf;
};

// Position tangents of the differentiable sampling mode: injected per
// nucleon ([n][A][4], [n][B][4]: dx/dR, dy/dR, dx/da, dy/da), written per
// nucleon in sorted order (ntan [n][A+B][4]) and per splat source
// (stan [n][max_src]).  All NULL when unused.
struct TangentIO {
  const double *inj_proj, *inj_targ;
  double *ntan;
  float4 *stan;
  // per event [n][4]: the orientations (cos theta, phi) of the projectile
  // and the target drawn by the accepted attempt (NULL: not written)
  double *orient;
};

// The parameters that differ between the systems of a mixed batch (the
// nuclei, sigma_in and its derived pairing constants, the impact-parameter
// range and the Npart cut).
struct SystemDev {
  NucleusDev nuc[2];
  double dsq, sigma_gg, sigin, bmin, bmax;
  int npmin, npmax;
};

// Per-context constants passed by value to every kernel.
struct DevParams {
  int nx, ny;
  double xmin, ymin, dx, dy;
  double inv_dx, inv_dy;   // 1 / dx, 1 / dy (the sources' grid offsets)
  double width, w2, quark_width, peak;   // nucleon width, width^2, 1/(2 pi w^2)
  double dsq, sigin, sigma_gg;
  double alpha, final_factor;
  int which_mc_model, sub_model, shape_of_nucleons, shape_of_entropy, collision_criterion;
  int npmin, npmax;
  double bmin, bmax;
  NucleusDev nuc[2];
  uint64_t seed;
  int max_attempts, max_coll, max_src;
  int ecc_from, ecc_to;
  int kln_tmax;
  double kln_dT;
  float kln_dT_f;           // (float)kln_dT
  float kln_inv_dT_f;       // (float)(1 / kln_dT), read per cell
  // bound on the relative error of a term of the splats' FP32 thickness sums
  // against the reference's FP64 terms (a cell whose T/dT lies within the
  // event's bound of an integer takes its table cell from FP64 sums), and
  // half the smallest nonzero thickness a source adds (its value at the cut)
  float kln_band, kln_tzero;
  const float *kln_table;   // [tmax][tmax] (device)
  // the six-point interpolation of each table cell (i, j) as polynomial
  // coefficients (axx, axy, ayy, bx, by, v00, 0, 0), from the FP64 table
  const float4 *kln_coef;   // [tmax][tmax][2] (device)
  int want_ta, want_tb;     // thickness planes requested
  int splat_mw;             // widest splat window in columns (+ margin)
  int n_planes;             // accumulator planes of the splat (1..3)
  int no_moments;           // skip the eccentricity pass (averaged mode)
  int want_spect;           // spectator records (averaged mode's spectator densities)
  int want_binary;          // binary-collision records whatever the model (rho_binary)
  // multiplicity fluctuations (cc_fluctuation_model 6): Gamma(k, theta)
  // weights per participant and per binary collision
  int fluct;
  double fluct_k_part, fluct_th_part, fluct_k_coll, fluct_th_coll;
  // per-cell negative-binomial fluctuations (cc_fluctuation_model 1, 2):
  // k = nbd_k (model 1) or nbd_kpp min(T_A, T_B) sigma_in / 10 (model 2)
  int nbd;
  double nbd_k, nbd_kpp;
};

// Which events a persistent CTA takes.  Static: blockIdx.x, + gridDim.x, ...
// Dynamic (next != NULL): a ticket from the counter *next (zeroed before the
// launch) per event, so that CTAs that finish early take more; with order,
// ticket k is event order[k] (the heaviest first).  Every event's result is
// independent of which CTA computes it.
struct EventQueue {
  const int *order;
  int *next;
};
__device__ __forceinline__ int queue_first(const EventQueue &q, int *s_k) {
  if (!q.next) return blockIdx.x;
  __syncthreads();   // every thread has read the previous ticket
  if (threadIdx.x == 0) *s_k = atomicAdd(q.next, 1);
  __syncthreads();
  return *s_k;
}
__device__ __forceinline__ int queue_next(const EventQueue &q, int k, int *s_k) {
  return q.next ? queue_first(q, s_k) : k + (int)gridDim.x;
}
__device__ __forceinline__ int queue_event(const EventQueue &q, int k) { return q.order ? q.order[k] : k; }

// Averaged mode: an event's frame, the centre of mass (x, y) and the
// rotation (cos, sin) that brings its participant plane to the x axis.
struct alignas(16) AvgFrame {
  double x, y, c, s;
};

// Per-event record written by the sampling/pairing stage.
struct EventRec {
  double b;
  int npart1, npart2, ncoll, nsrc;
  int attempts, status;
  int imin, imax, jmin, jmax;   // bounding box of all splat windows (grid idx)
  int nsplat;                   // records [0, nsplat) hold every splat source
  unsigned long long ev;        // global event id (keys the per-cell fluctuation streams)
};

// ---------------------------------------------------------------- Philox
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}

__host__ __device__ __forceinline__ double u53(uint32_t lo, uint32_t hi) {
  uint64_t v = ((uint64_t)hi << 32) | lo;
  return ((double)(v >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// (float)u53(lo, hi) with integer operations only: the value (m + 1/2) 2^-53,
// m the top 53 bits of (hi, lo), rounded to double and then to float (each
// to nearest, ties to even), as the FP64 expression (float)u53 rounds it.
__host__ __device__ __forceinline__ float u53f(uint32_t lo, uint32_t hi) {
  const uint64_t m = (((uint64_t)hi << 32) | lo) >> 11;
  uint64_t x = 2 * m + 1;   // the value is x 2^e
  int e = -54;
  if (x >> 53) {            // 54 significant bits: the double drops the last one (a tie) to even
    const uint64_t h = x >> 1;
    x = h + (h & 1);
    e = -53;
  }
#ifdef __CUDA_ARCH__
  const int msb = 63 - __clzll((long long)x);
#else
  const int msb = 63 - __builtin_clzll(x);
#endif
  if (msb > 23) {           // to 24 significant bits
    const int sh = msb - 23;
    uint64_t q = x >> sh;
    const uint64_t rem = x & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    x = q;
    e += sh;
  }
  const uint32_t bits = (uint32_t)(e + 127) << 23;   // 2^e, a normal float (e >= -54)
  float scale;
#ifdef __CUDA_ARCH__
  scale = __int_as_float((int)bits);
#else
  __builtin_memcpy(&scale, &bits, sizeof(scale));
#endif
  return (float)(uint32_t)x * scale;   // x <= 2^24: exact
}

// Two uniforms in (0,1): counter {slot, stream, event_lo, event_hi},
// key {seed_lo, seed_hi}.
__host__ __device__ __forceinline__ void uniform2(uint64_t seed, uint64_t event, uint32_t stream,
                                                  uint32_t slot, double &u0, double &u1) {
  uint32_t c[4] = {slot, stream, (uint32_t)event, (uint32_t)(event >> 32)};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  u0 = u53(c[0], c[1]);
  u1 = u53(c[2], c[3]);
}

// uniform2 rounded to float, without FP64 arithmetic
__host__ __device__ __forceinline__ void uniform2f(uint64_t seed, uint64_t event, uint32_t stream, uint32_t slot,
                                                   float &u0, float &u1) {
  uint32_t c[4] = {slot, stream, (uint32_t)event, (uint32_t)(event >> 32)};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  u0 = u53f(c[0], c[1]);
  u1 = u53f(c[2], c[3]);
}

enum StreamId : uint32_t {
  ST_EVENT = 0, ST_PROJ = 1, ST_TARG = 2, ST_DEUT = 3, ST_COLL = 4, ST_FLUCT = 5, ST_NBD = 6, ST_CONF = 7
};
__host__ __device__ __forceinline__ uint32_t stream_id(int attempt, uint32_t sid) {
  return ((uint32_t)attempt << 8) | sid;
}

#ifdef __CUDACC__
// Gamma(k, theta) from counters base + 2t, base + 2t + 1 (t < 15) and, for
// k < 1, base + 31 of a Philox stream: the method of Marsaglia and Tsang
// ("A simple method for generating gamma variables", ACM TOMS 26 (2000)
// 363) with Gamma(k) = Gamma(k+1) U^(1/k) for k < 1 and Box-Muller normals.
static __device__ inline double gamma_philox(uint64_t seed, uint64_t ev, uint32_t sid, uint32_t base, double k,
                                      double theta) {
  const double kk = k < 1 ? k + 1 : k;
  const double d = kk - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  double g = d;   // after 15 rejections (probability below 1e-19)
  for (int t = 0; t < 15; t++) {
    double u0, u1, w0, w1;
    uniform2(seed, ev, sid, base + 2 * t, u0, u1);
    uniform2(seed, ev, sid, base + 2 * t + 1, w0, w1);
    const double x = sqrt(-2.0 * log(1.0 - u0)) * cos(2.0 * M_PI * u1);
    double v = 1.0 + c * x;
    if (v <= 0) continue;
    v = v * v * v;
    if (log(1.0 - w0) < 0.5 * x * x + d - d * v + d * log(v)) {
      g = d * v;
      break;
    }
  }
  if (k < 1) {
    double u0, u1;
    uniform2(seed, ev, sid, base + 31, u0, u1);
    g *= pow(1.0 - u0, 1.0 / k);
  }
  return g * theta;
}

// Poisson(lambda) from counters base, base + 1, ... (< 32): inversion below
// lambda = 10, else the transformed rejection with squeeze of Hoermann
// ("The transformed rejection method for generating Poisson random
// variables", Insurance: Mathematics and Economics 12 (1993) 39).
static __device__ inline double poisson_philox(uint64_t seed, uint64_t ev, uint32_t sid, uint32_t base, double lam) {
  if (!(lam > 0)) return 0;
  if (lam < 10) {
    double u, unused;
    uniform2(seed, ev, sid, base, u, unused);
    double p = exp(-lam), s = p;
    int n = 0;
    while (u > s && n < 1000) {
      n++;
      p *= lam / n;
      s += p;
    }
    return n;
  }
  const double slam = sqrt(lam), loglam = log(lam);
  const double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
  const double invalpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2);
  for (int t = 0; t < 32; t++) {
    double U, V;
    uniform2(seed, ev, sid, base + t, U, V);
    U -= 0.5;
    const double us = 0.5 - fabs(U);
    const double kf = floor((2 * a / us + b) * U + lam + 0.43);
    if (us >= 0.07 && V <= vr) return kf;
    if (kf < 0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + kf * loglam - lgamma(kf + 1)) return kf;
  }
  return floor(lam + 0.5);   // after 32 rejections (probability below 1e-30)
}

// MCnucl::fluctuateCurrentDensity (src/MCnucl.cpp:869-905): the cell's
// density v becomes n/(dx dy), n negative-binomial with mean nb = v dx dy
// and shape k (NBD::rand(nb/(nb+k), k)), drawn as Poisson(Gamma(k, nb/k))
// from the cell's stream (stream 6, counters 64 cell + ...).  t1, t2: T_A,
// T_B of the cell (model 2).
static __device__ __noinline__ float nbd_cell(const DevParams &P, uint64_t ev, uint32_t cell, float v, float t1, float t2) {
  const double area = P.dx * P.dy, nb = (double)v * area;
  double k = P.nbd_k;
  if (P.nbd == 2) {
    k = P.nbd_kpp * fmin((double)t1, (double)t2) * P.sigin / 10;
    if (nb < 1e-10) return v;   // left as it is (MCnucl.cpp:893-895)
  }
  if (!(nb > 0) || !(k > 0)) return 0.f;   // NBD::rand is 0 for p = 0 or p = 1
  const uint32_t sid = stream_id(0, ST_NBD);
  const double lam = gamma_philox(P.seed, ev, sid, 64 * cell, k, nb / k);
  return (float)(poisson_philox(P.seed, ev, sid, 64 * cell + 32, lam) / area);
}
#endif

// ------------------------------------------------------- exact helpers
#ifdef __CUDACC__
// A position in grid units split into its cell (exact in FP32) and the
// fraction within it, (v - vmin)/d - cell, from the FP64 position: the FP32
// distance (k - cell) - fraction from the position to grid point k then errs
// by at most 2^-25 + 2^-24 |distance| grid units, where a difference of FP32
// coordinates errs by 2^-24 of the coordinates' magnitude.
__device__ __forceinline__ void grid_offset(double v, double vmin, double inv_d, float &cell, float &frac) {
  // a product by the rounded 1/d: within an FP64 ulp or two of the quotient,
  // far below the FP32 rounding of the fraction (an FP64 division costs
  // several times more on this part)
  const double g = (v - vmin) * inv_d;
  const double c = floor(g);
  cell = (float)c;
  frac = (float)(g - c);
}
__device__ __forceinline__ void set_grid_offsets(Source &s, const DevParams &P) {
  grid_offset(s.x, P.xmin, P.inv_dx, s.gi0, s.gfx);
  grid_offset(s.y, P.ymin, P.inv_dy, s.gj0, s.gfy);
}
#endif

// (int)((v - mn)/d) as the reference computes it in FP64 (C++ truncation
// toward zero).  FP64 division is slow on this part, so the FP32 estimate
// is used whenever it is provably on the same side of every integer.
__device__ __forceinline__ int trunc_index(double v, double mn, double d, float inv_d) {
  float t = (float)(v - mn) * inv_d;      // |error| < ~4e-5 for |t| < 400
  float f = floorf(t);
  float fr = t - f;
  if (fr > 1e-3f && fr < 1.f - 1e-3f) {
    int i = (int)f;
    // truncation toward zero differs from floor for negative non-integers
    return (t < 0.f) ? i + 1 : i;
  }
  double e = __ddiv_rn(__dadd_rn(v, -mn), d);
  return (int)e;
}

// exact FP64 distance tests with explicit rounding (no contraction)
__device__ __forceinline__ double sq_dist_rn(double x1, double y1, double x2, double y2) {
  double dx = __dadd_rn(x2, -x1), dy = __dadd_rn(y2, -y1);
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

}  // namespace smc
