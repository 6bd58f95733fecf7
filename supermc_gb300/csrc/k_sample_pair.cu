// Stage 1 of the event pipeline: nucleus sampling, participant/binary
// pairing and construction of the splat sources, one CTA per event.
//
// Reference behaviour restated here:
//   impact parameter and retry loop   src/MakeDensity.cpp:2147-2162
//   Woods-Saxon sampling, hard core   src/Nucleus.cpp:187-317, :578-621
//   deuteron (Hulthen)                src/Nucleus.cpp:342-359, src/HulthenFunc.cpp:27-41
//   pairing (disk / Gaussian)         src/MCnucl.cpp:217-385
//   binary-collision midpoints        src/MCnucl.cpp:326-352
//   splat windows                     src/MCnucl.cpp:432-478, :688-779, :822-866
//   eccentricity hot-spot region      src/MCnucl.cpp:1303-1323, src/MakeDensity.cpp:2341-2359
#include "smc_device.cuh"
#include "smc_kernels.h"

#include <cfloat>
#include <climits>

namespace smc {

constexpr int kNT = 256;   // threads per CTA; also the candidate batch size
constexpr int kSlab = 32;  // z slabs of the hard-core search, at most
static_assert(kMaxA <= kNT, "one nucleon per thread");
static_assert(kMaxA % 4 == 0, "float4 rows");

// Per-event constants, derived once by thread 0 from the event's parameters
// (FP64 work is costly here: the other threads read the results)
struct SampleConsts {
  double cbox, d_max, disk_val_d;   // participant box half width 4 max(w, w_q), splat radius, 10 / sigma_in
  float cbox_f, d_max_f, xmin_f, ymin_f;
  float dsq_lo, dsq_hi, hit_rad;    // FP32 disk-test thresholds, with margins
  float peak, disk_val, wn;         // FP32 peak, 10 / sigma_in, (1 - alpha) / 2
  float box_lim, w2, sigma_gg;      // FP32 copies for the pair tests
  int swept;
  // eccentricity region of the event
  double rxl, ryl;
  float rxl_f, ryl_f;
  int nXp, nYp, ioff, joff;
};

// Working memory of the Woods-Saxon sampler for a group of NT threads (the
// whole CTA, or half of it when the two nuclei are sampled at once)
template <int NT>
struct alignas(16) SampStore {
  // candidate batch (nucleus frame): x, y, z; before the direction is drawn
  // (r, candidate index bits, 0, 0)
  float4 cpos[NT];
  union {
    uint32_t cmask[NT][NT / 32];           // earlier batch candidates each one conflicts with
    float4 spos[kMaxA];                    // accepted nucleons ordered by z slab
  } u;
  uint32_t smask[kSlab][NT / 32];          // hard-core survivors of the batch per z slab
  int slab_cnt[kSlab], slab_cur[kSlab], slab_start[kSlab + 1];
  uint8_t cslab[NT];                       // z slab of each batch candidate
  uint32_t vb[NT / 32];                    // hard-core survivors
  uint32_t keep[NT / 32], conf[NT / 32];   // batch resolution state: kept, undecided
  int ired[NT / 32];                       // radially accepted candidates per warp
  static_assert(kSlab * (NT / 32) == NT, "one slab-mask word per thread is cleared");
};

struct alignas(16) SampleSmem {
  union {
    SampStore<kNT> full;         // one nucleus at a time, all threads
    SampStore<kNT / 2> half[2];  // both nuclei at once, one per half
  } samp;
  // read four at a time (float4): 16-byte aligned rows of kMaxA (a multiple of 4)
  alignas(16) float ax[2][kMaxA];
  alignas(16) float ay[2][kMaxA];
  alignas(16) float az[2][kMaxA];            // accepted (nucleus frame)
  double X[2][kMaxA], Y[2][kMaxA];           // final positions, sorted by x
  alignas(16) float Xf[2][kMaxA];
  float Yf[2][kMaxA];
  int hits[2][kMaxA];
  int scan[32];
  double red[kNT / 32 * 3];
  float2 red2[kNT / 32 * 2];
  int ired[kNT / 32 * 4];
  double red4[kNT / 32];
  double bmean[2];   // block means broadcast by block_mean2_f
  long long lred[32];
  double b;
  double ori[2][2];   // nucleus orientations (cos theta, phi) of the attempt
  int cfg_idx[2];     // configuration of each table nucleus
  SampleConsts sc;
};

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ float sph2(float ct) { return (3.0f * ct * ct - 1.0f) * 0.31539156525252005f; }
__device__ __forceinline__ float sph4(float ct) {
  float c2 = ct * ct;
  return (35.0f * c2 * c2 - 30.0f * c2 + 3.0f) * 0.10578554691520431f;
}

// Point3D::rotate (src/MathBasics.cpp:41-50), FP64
__device__ __forceinline__ void rotate3d(double &x, double &y, double &z, double cth, double phi) {
  double sphi, cphi;
  sincos(phi, &sphi, &cphi);
  const double sth = sqrt(fmax(0.0, 1.0 - cth * cth));
  const double x0 = x, y0 = y, z0 = z;
  x = cth * cphi * x0 - sphi * y0 + sth * cphi * z0;
  y = cth * sphi * x0 + cphi * y0 + sth * sphi * z0;
  z = -sth * x0 + cth * z0;
}

// Point3D::rotate (src/MathBasics.cpp:41-50)
__device__ __forceinline__ void rotate3f(float &x, float &y, float &z, float cth, float phi) {
  float sphi, cphi;
  sincosf(phi, &sphi, &cphi);
  float sth = sqrtf(fmaxf(0.f, 1.f - cth * cth));
  float x0 = x, y0 = y, z0 = z;
  x = cth * cphi * x0 - sphi * y0 + sth * cphi * z0;
  y = cth * sphi * x0 + cphi * y0 + sth * sphi * z0;
  z = -sth * x0 + cth * z0;
}

// ---------------------------------------------- inverse-CDF radii
// Differentiable sampling mode (no reference counterpart; the reference
// samples radii by rejection, src/Nucleus.cpp:578-621): r solves
// N(r) = u N(rmax), N(r) = int_0^r t^2 rho(t) dt for the reference's
// truncated density rho = 1/(1+exp((r-R)/a)), r <= rmax = R + 2.5.  N and
// its R, a derivatives are tabulated on the host; between nodes they are
// cubic Hermite interpolants whose end-point slopes are the exact integrands.

// r^2 rho(r) and its derivatives in R and a
__device__ __forceinline__ void ws_weights(const NucleusDev &n, double r, double &f, double &fR, double &fa) {
  const double rho = 1.0 / (1.0 + exp((r - n.R) / n.a));
  const double d = rho * (1.0 - rho) / n.a;
  f = r * r * rho;
  fR = r * r * d;
  fa = fR * (r - n.R) / n.a;
}

// cubic Hermite interpolant on [r_k, r_k + h] at t in [0, 1] from the end
// values y0, y1 and slopes (per unit r) f0, f1
__device__ __forceinline__ double hermite(double t, double h, double y0, double y1, double f0, double f1) {
  const double t2 = t * t, t3 = t2 * t;
  return (2 * t3 - 3 * t2 + 1) * y0 + (t3 - 2 * t2 + t) * h * f0 + (3 * t2 - 2 * t3) * y1 + (t3 - t2) * h * f1;
}

// the radius for the uniform u: bisection over the table, then Newton
// steps on the interval's interpolant (monotone: N increases with r)
__device__ double icdf_radius(const NucleusDev &n, double u) {
  const double *N = n.icdf;
  const double T = u * n.icdf_ntot;
  // N[lo] <= T < N[hi], starting from the bucket of u
  const double *start = N + 3 * (size_t)n.icdf_m;
  const int b = min((int)(u * n.icdf_nb), n.icdf_nb - 1);
  int lo = (int)start[b], hi = min((int)start[b + 1] + 1, n.icdf_m - 1);
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (N[mid] <= T) lo = mid;
    else hi = mid;
  }
  const double h = n.icdf_h, r0 = lo * h;
  double f0, f1, g0, g1;
  ws_weights(n, r0, f0, g0, g1);
  ws_weights(n, r0 + h, f1, g0, g1);
  const double y0 = N[lo], y1 = N[lo + 1];
  double t = y1 > y0 ? (T - y0) / (y1 - y0) : 0.0;
  for (int it = 0; it < 6; it++) {   // quadratic convergence from the linear guess
    const double t2 = t * t;
    const double p = hermite(t, h, y0, y1, f0, f1) - T;
    const double dp =
        (6 * t2 - 6 * t) * y0 + (3 * t2 - 4 * t + 1) * h * f0 + (6 * t - 6 * t2) * y1 + (3 * t2 - 2 * t) * h * f1;
    if (!(dp > 0)) break;
    t = fmin(fmax(t - p / dp, 0.0), 1.0);
  }
  return r0 + t * h;
}

// (dr/dR)/r and (dr/da)/r at the radius r (implicit differentiation of
// F(r) = N(r)/N(rmax) = u):  dr/dp = -(N_p(r) - F(r) dN(rmax)/dp) / (r^2 rho(r))
__device__ void icdf_tangent(const NucleusDev &n, double r, double &sR, double &sa) {
  sR = sa = 0.0;
  if (!(r > 1e-9)) return;
  const int m = n.icdf_m;
  const double h = n.icdf_h;
  const int k = min((int)(r / h), m - 2);
  const double t = fmin((r - k * h) / h, 1.0);
  double f0, fR0, fa0, f1, fR1, fa1, f, fR, fa;
  ws_weights(n, k * h, f0, fR0, fa0);
  ws_weights(n, (k + 1) * h, f1, fR1, fa1);
  ws_weights(n, r, f, fR, fa);
  const double *N = n.icdf, *NR = N + m, *Na = NR + m;
  const double F = hermite(t, h, N[k], N[k + 1], f0, f1) / n.icdf_ntot;
  const double nR = hermite(t, h, NR[k], NR[k + 1], fR0, fR1);
  const double na = hermite(t, h, Na[k], Na[k + 1], fa0, fa1);
  if (!(f > 0)) return;
  sR = -(nR - F * n.icdf_dntot_R) / (f * r);
  sa = -(na - F * n.icdf_dntot_a) / (f * r);
}

// One Woods-Saxon candidate from four uniforms (Nucleus::getDeformRandomWS)
// (u0..u3 rounded to float; u0d the FP64 u0, read only by inverse-CDF radii).
// Spherical nuclei: the radius and its acceptance come from u0, u1 alone
// (ws_radius), the direction from u2, u3 (ws_direction); deformed nuclei
// need all four for the acceptance (ws_candidate_deformed).
__device__ __forceinline__ bool ws_radius(const NucleusDev &n, double u0d, float u0, float u1, float &r) {
  if (n.icdf) {   // every candidate passes the radial step
    r = (float)icdf_radius(n, u0d);
    return true;
  }
  r = n.rmax_f * powf(u0, 1.0f / 3.0f);
  return !(u1 * n.rw_max_f > 1.0f / (1.0f + expf((r - n.R_f) / n.a_f)));
}

__device__ __forceinline__ void ws_direction(float r, float u2, float u3, float &x, float &y, float &z) {
  float cx = 1.0f - 2.0f * u2;
  float sx = sqrtf(fmaxf(0.f, 1.0f - cx * cx));
  float sp, cp;
  sincospif(2.0f * u3, &sp, &cp);
  x = r * sx * cp; y = r * sx * sp; z = r * cx;
}

__device__ __forceinline__ bool ws_candidate_deformed(const NucleusDev &n, float ctr, float phir, float u0, float u1,
                                                      float u2, float u3, float &x, float &y, float &z) {
  const float R = n.R_f, a = n.a_f;
  const float r = n.rmax_f * powf(u0, 1.0f / 3.0f);
  float cx = 1.0f - 2.0f * u1;
  float rad1 = R * (1.0f + n.beta2_f * sph2(cx) + n.beta4_f * sph4(cx));
  float rw1 = 1.0f / (1.0f + expf(-rad1 / a));
  if (u2 * rw1 > 1.0f / (1.0f + expf((r - rad1) / a))) return false;
  float sx = sqrtf(fmaxf(0.f, 1.0f - cx * cx));
  float sp, cp;
  sincospif(2.0f * u3, &sp, &cp);
  x = r * sx * cp; y = r * sx * sp; z = r * cx;
  rotate3f(x, y, z, ctr, phir);
  return true;
}

// HulthenFunc::CDF (src/HulthenFunc.cpp:27-36)
__device__ double hulthen_cdf(double r) {
  const double alpha = .228, beta = 1.18;
  if (r <= 0) return 0;
  const double c = (alpha * beta * (alpha + beta)) / ((alpha - beta) * (alpha - beta));
  return 2 * c * (2 * (exp(-r * (alpha + beta)) / (alpha + beta)) - .5 * exp(-2 * alpha * r) / alpha -
                  .5 * exp(-2 * beta * r) / beta + .5 / alpha + .5 / beta - 2 / (alpha + beta));
}
// invertFunc Newton iteration as used by HulthenFunc::invCDF (src/arsenal.cpp:318-387)
__device__ double hulthen_inv(double y) {
  const double xL = 0, xR = 100.0, dx = 0.001, acc = 0.001 * 0.001;
  double XX2 = 1.0, XX1 = XX2 - 10 * acc;
  for (int it = 0; it < 61 && fabs(XX2 - XX1) > acc; it++) {
    XX1 = XX2;
    double F0 = hulthen_cdf(XX1) - y;
    double X1 = (XX1 > xL + dx) ? XX1 - dx : xL;
    double X2 = (XX1 < xR - dx) ? XX1 + dx : xR;
    double F3 = (hulthen_cdf(X1) - hulthen_cdf(X2)) / (X1 - X2);
    XX2 = XX1 - F0 / F3;
  }
  return XX2;
}

// Means over the block of two FP32 values per thread, (sum v0) / n and
// (sum v1) / n, exact to double precision for the sums that occur here:
// double-float warp sums, then the FP64 additions and division of each sum
// by one lane (FP64 throughput is a small fraction of FP32 here), broadcast
// through shared memory.
__device__ __forceinline__ void block_mean2_f(float v0, float v1, int n, float2 *red, double *out, double &m0,
                                              double &m1) {
  float hi[2] = {v0, v1}, lo[2] = {0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 2; k++)
    for (int o = 16; o; o >>= 1) {
      float bh = __shfl_xor_sync(0xffffffffu, hi[k], o), bl = __shfl_xor_sync(0xffffffffu, lo[k], o);
      float s2 = hi[k] + bh, bb = s2 - hi[k];
      float e = (hi[k] - (s2 - bb)) + (bh - bb) + (lo[k] + bl);
      hi[k] = s2 + e;
      lo[k] = e - (hi[k] - s2);
    }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[w] = make_float2(hi[0], lo[0]);
    red[kNT / 32 + w] = make_float2(hi[1], lo[1]);
  }
  __syncthreads();
  if (threadIdx.x < 2) {   // lane k: sum k
    const float2 *rk = red + threadIdx.x * (kNT / 32);
    double sk = 0;
    for (int i = 0; i < kNT / 32; i++) sk += (double)rk[i].x + (double)rk[i].y;
    out[threadIdx.x] = sk / n;
  }
  __syncthreads();
  m0 = out[0];
  m1 = out[1];
}

// three block sums with one barrier (red: 3 * kNT / 32 ints)
__device__ __forceinline__ void block_sum3_i(int a, int b, int c, int *red, int &sa, int &sb, int &sc) {
  for (int o = 16; o; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[w] = a;
    red[kNT / 32 + w] = b;
    red[2 * (kNT / 32) + w] = c;
  }
  __syncthreads();
  sa = sb = sc = 0;
  for (int i = 0; i < kNT / 32; i++) {
    sa += red[i];
    sb += red[kNT / 32 + i];
    sc += red[2 * (kNT / 32) + i];
  }
}

// Samples one nucleus into sm.ax/ay/az[w] (nucleus frame, centre of mass
// not yet removed).  Candidates are consumed in order; a candidate is kept
// iff it passes the radial test and lies at least d_min from every nucleon
// kept before it -- the sequential rule of Nucleus::populate, evaluated a
// batch of kNT candidates at a time.  Returns false if the candidate cap is hit.
//
// Per batch: the radially accepted candidates are compacted (nv of them)
// and, for spherical nuclei, only these draw their direction.  Distances
// are tested only between neighbouring z slabs: the slabs are at least
// 1.01 d_min thick, so points two or more slabs apart are farther than
// d_min apart even after rounding.  Each candidate is tested against the
// nucleons accepted so far (held ordered by slab, rebuilt every batch), then
// against the earlier valid candidates of the batch in 32x32 blocks spread
// over the warps, giving a bit row per candidate.  Candidates without
// conflicts are kept; the conflicted ones are decided by warp 0 in rounds:
// a candidate is dropped once an earlier conflicting candidate is kept and
// kept once all of them are dropped (the earliest undecided one is decided
// every round, so the rounds end).  This reproduces the sequential rule.
// the sampler's barriers: the CTA's, or a named barrier of one half
struct FullSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct HalfSync {
  int h;
  __device__ __forceinline__ void operator()() const {
    if (h == 0) asm volatile("bar.sync 1, %0;" ::"n"(kNT / 2) : "memory");
    else asm volatile("bar.sync 2, %0;" ::"n"(kNT / 2) : "memory");
  }
};

template <int NT, typename Sync>
__device__ bool sample_ws(SampleSmem &sm, SampStore<NT> &ss, const NucleusDev &n, int w, uint64_t seed, uint64_t ev,
                          int attempt, float ctr, float phir, Sync sync) {
  const int tid = threadIdx.x & (NT - 1), lane = tid & 31, wid = tid >> 5;
  const int A = n.A;
  const float dmin2 = n.dmin2_f;
  const uint32_t sid = stream_id(attempt, w == 0 ? ST_PROJ : ST_TARG);
  // z slabs over [-rmax, rmax]: nslab of them, each at least 1.01 d_min thick
  const float rmax = n.rmax_f, inv_w = n.slab_inv_w;
  const int nslab = n.nslab;
  auto slab_of = [&](float z) { return min(nslab - 1, max(0, (int)floorf((z + rmax) * inv_w))); };
  if (tid < kSlab) { ss.slab_cnt[tid] = 0; ss.slab_cur[tid] = 0; }
  sync();
  int n_acc = 0;
  // A batch goes on with the first `cap` radially accepted candidates, a few
  // more than the nucleons still missing (the hard core rejects a few per
  // cent): a batch that reaches its cap ends at its last valid candidate and
  // the next one starts after it, so every candidate is decided once and in
  // order whatever the batch (a small nucleus's batch then carries about as
  // many candidates as it needs, not the whole group's worth).
  for (uint32_t base = 0; n_acc < A;) {
    if (base > (1u << 20)) return false;
    const int need = A - n_acc;
    const int cap = min(NT, need + need / 8 + 8);
    const uint32_t c = base + tid;
    float u0, u1;
    uniform2f(seed, ev, sid, 2 * c, u0, u1);
    float x = 0.f, y = 0.f, z = 0.f, r = 0.f;
    bool ws;
    if (n.deformed) {
      float u2, u3;
      uniform2f(seed, ev, sid, 2 * c + 1, u2, u3);
      ws = ws_candidate_deformed(n, ctr, phir, u0, u1, u2, u3, x, y, z);
    } else {
      double u0d = 0, unused;
      if (n.icdf) uniform2(seed, ev, sid, 2 * c, u0d, unused);
      ws = ws_radius(n, u0d, u0, u1, r);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, ws);
    if (lane == 0) ss.ired[wid] = __popc(bal);
    // accepted nucleons per slab
    for (int k = tid; k < n_acc; k += NT) atomicAdd(&ss.slab_cnt[slab_of(sm.az[w][k])], 1);
    ss.smask[tid / (NT / 32)][tid & (NT / 32 - 1)] = 0u;   // kSlab * NT / 32 == NT words
    sync();
    // the radially accepted candidates, compacted in candidate order; the
    // accepted nucleons ordered by slab
    int off = 0, nv = 0;
#pragma unroll
    for (int q = 0; q < NT / 32; q++) {
      const int cq = ss.ired[q];
      off += q < wid ? cq : 0;
      nv += cq;
    }
    if (ws) {
      // the candidate number rides in w (the direction's stream slot, the
      // end of a capped batch)
      const int v = off + __popc(bal & ((1u << lane) - 1u));
      if (v < cap)
        ss.cpos[v] = n.deformed ? make_float4(x, y, z, __uint_as_float(c)) : make_float4(r, 0.f, 0.f, __uint_as_float(c));
    }
    // where the next batch starts (cpos[cap - 1].w is read after the batch's
    // last barrier, before the next batch writes cpos)
    const bool capped = nv > cap;
    nv = min(nv, cap);
    if (tid <= nslab) {
      int st = 0;
      for (int t = 0; t < tid; t++) st += ss.slab_cnt[t];
      ss.slab_start[tid] = st;
    }
    for (int k = tid; k < n_acc; k += NT) {
      const float ax = sm.ax[w][k], ay = sm.ay[w][k], az = sm.az[w][k];
      const int sl = slab_of(az);
      int st = 0;
      for (int t = 0; t < sl; t++) st += ss.slab_cnt[t];
      ss.u.spos[st + atomicAdd(&ss.slab_cur[sl], 1)] = make_float4(ax, ay, az, 0.f);
    }
    sync();
    // candidate tid (< nv): its direction, then the hard core against the
    // accepted nucleons of the neighbouring slabs
    bool ok = tid < nv;
    int sl = 0;
    if (ok) {
      const float4 p = ss.cpos[tid];
      if (n.deformed) {
        x = p.x; y = p.y; z = p.z;
      } else {
        float u2, u3;
        uniform2f(seed, ev, sid, 2 * __float_as_uint(p.w) + 1, u2, u3);
        ws_direction(p.x, u2, u3, x, y, z);
        ss.cpos[tid] = make_float4(x, y, z, p.w);
      }
      sl = slab_of(z);
      const int k1 = ss.slab_start[min(nslab, sl + 2)];
      for (int k = ss.slab_start[max(0, sl - 1)]; k < k1; k++) {
        const float4 a = ss.u.spos[k];
        const float dx = x - a.x, dy = y - a.y, dz = z - a.z;
        if (dx * dx + dy * dy + dz * dz < dmin2) { ok = false; break; }
      }
      ss.cslab[tid] = (uint8_t)sl;
    }
    const unsigned vb = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) {
      ss.vb[wid] = vb;
      ss.conf[wid] = 0u;
    }
    if (ok) atomicOr(&ss.smask[sl][wid], 1u << lane);
    sync();
    // conflicts with earlier valid candidates of the batch (neighbouring
    // slabs): block (q, r) holds later candidates q*32+lane against earlier
    // ones r*32+kk
    const int Q = (nv + 31) >> 5;
    for (int blk = wid; blk < Q * (Q + 1) / 2; blk += NT / 32) {
      int q = 0, s0 = 0;
      while (s0 + q + 1 <= blk) { s0 += q + 1; q++; }
      const int r = blk - s0, cq = q * 32 + lane;
      uint32_t bits = 0;
      if ((ss.vb[q] >> lane) & 1u) {
        const float4 pc = ss.cpos[cq];
        const int sc = ss.cslab[cq];
        uint32_t m = ss.smask[sc][r];
        if (sc > 0) m |= ss.smask[sc - 1][r];
        if (sc + 1 < nslab) m |= ss.smask[sc + 1][r];
        if (r == q) m &= (1u << lane) - 1u;
        while (m) {
          const int kk = __ffs(m) - 1;
          m &= m - 1u;
          const float4 pk = ss.cpos[r * 32 + kk];
          const float dx = pc.x - pk.x, dy = pc.y - pk.y, dz = pc.z - pk.z;
          if (dx * dx + dy * dy + dz * dz < dmin2) bits |= 1u << kk;
        }
      }
      ss.u.cmask[cq][r] = bits;
      const unsigned cf = __ballot_sync(0xffffffffu, bits != 0u);
      if (lane == 0 && cf) atomicOr(&ss.conf[q], cf);
    }
    sync();
    if (wid == 0) {
      // kept / undecided words (lane q < 8 owns word q)
      if (lane < NT / 32) {
        const uint32_t v = lane < Q ? ss.vb[lane] : 0u, u = lane < Q ? ss.conf[lane] : 0u;
        ss.keep[lane] = v & ~u;
        ss.conf[lane] = u;
      }
      __syncwarp();
      for (int round = 0; round < NT; round++) {
        uint32_t kw = lane < NT / 32 ? ss.keep[lane] : 0u, uw = lane < NT / 32 ? ss.conf[lane] : 0u;
        if (!__any_sync(0xffffffffu, uw != 0u)) break;
        for (int q = 0; q < Q; q++) {
          bool kept = false, decided = false;
          if ((ss.conf[q] >> lane) & 1u) {
            bool hit = false, pend = false;
            for (int r = 0; r <= q; r++) {
              const uint32_t m = ss.u.cmask[q * 32 + lane][r];
              hit |= (m & ss.keep[r]) != 0u;
              pend |= (m & ss.conf[r]) != 0u;
            }
            decided = hit || !pend;
            kept = !hit && !pend;
          }
          const unsigned kb = __ballot_sync(0xffffffffu, kept), db = __ballot_sync(0xffffffffu, decided);
          if (lane == q) { kw |= kb; uw &= ~db; }
        }
        __syncwarp();
        if (lane < NT / 32) { ss.keep[lane] = kw; ss.conf[lane] = uw; }
        __syncwarp();
      }
    }
    sync();
    // kept candidates in candidate order, up to the nucleons still missing
    {
      const uint32_t kw = ss.keep[wid];
      int before = 0, total = 0;
#pragma unroll
      for (int q = 0; q < NT / 32; q++) {
        const int pq = __popc(ss.keep[q]);
        before += q < wid ? pq : 0;
        total += pq;
      }
      before += __popc(kw & ((1u << lane) - 1u));
      if (((kw >> lane) & 1u) && n_acc + before < A) {
        const float4 p = ss.cpos[tid];
        sm.ax[w][n_acc + before] = p.x;
        sm.ay[w][n_acc + before] = p.y;
        sm.az[w][n_acc + before] = p.z;
      }
      n_acc += min(total, A - n_acc);
      if (tid < kSlab) { ss.slab_cnt[tid] = 0; ss.slab_cur[tid] = 0; }
    }
    sync();
    base = capped ? __float_as_uint(ss.cpos[cap - 1].w) + 1u : base + NT;
  }
  return true;
}

// Places nucleus w: nucleus-frame positions -> centre-of-mass removed in
// FP64 -> shifted by xc along x -> sorted by x (the reference sorts by the
// left box edge x-4w, src/Nucleus.cpp:314, the same order).
// With cfg (a light nucleus's configuration, [A][3]) the positions are the
// configuration rotated by (cth, phi) in FP64 and shifted by xc, not
// recentred (src/Nucleus.cpp:210-236, 555-574).
// With ntan (this nucleus's [A][4] rows of the per-nucleon tangents) the
// position tangents follow the same order: injected ones as given, those
// of inverse-CDF radii as (dr/dp)/r times the nucleus-frame point minus
// their mean over the nucleus (the centre-of-mass shift), else zero.
__device__ void place_sorted(SampleSmem &sm, int w, int A, double xc, const double *inj_xy,
                             const NucleusDev &nu, const double *inj_tan, double *ntan,
                             const double *cfg = nullptr, double cth = 1.0, double phi = 0.0) {
  const int tid = threadIdx.x;
  double px = 0, py = 0;
  float rx = 0.f, ry = 0.f;
  float tg[4] = {0.f, 0.f, 0.f, 0.f};
  if (ntan && inj_xy && inj_tan && tid < A)
    for (int c = 0; c < 4; c++) tg[c] = (float)inj_tan[4 * tid + c];
  if (ntan && !inj_xy && !cfg && nu.icdf && !nu.deformed && A > 2) {
    double sR = 0, sa = 0;
    float x = 0.f, y = 0.f;
    if (tid < A) {
      x = sm.ax[w][tid];
      y = sm.ay[w][tid];
      const float z = sm.az[w][tid];
      icdf_tangent(nu, sqrt((double)x * x + (double)y * y + (double)z * z), sR, sa);
    }
    float v[4] = {(float)(sR * x), (float)(sR * y), (float)(sa * x), (float)(sa * y)};
    for (int c = 0; c < 4; c += 2) {
      double m0, m1;
      block_mean2_f(tid < A ? v[c] : 0.f, tid < A ? v[c + 1] : 0.f, A, sm.red2, sm.bmean, m0, m1);
      __syncthreads();
      tg[c] = (float)(v[c] - m0);
      tg[c + 1] = (float)(v[c + 1] - m1);
    }
  }
  if (inj_xy) {
    if (tid < A) { px = inj_xy[2 * tid]; py = inj_xy[2 * tid + 1]; }
  } else if (cfg) {
    if (tid < A) {
      double x = cfg[3 * tid], y = cfg[3 * tid + 1], z = cfg[3 * tid + 2];
      rotate3d(x, y, z, cth, phi);
      px = x + xc;
      py = y;
      rx = (float)x;
      ry = (float)y;
    }
  } else {
    double mxa, mya;   // centre of mass (block_mean2_f ends with a barrier)
    block_mean2_f(tid < A ? sm.ax[w][tid] : 0.f, tid < A ? sm.ay[w][tid] : 0.f, A, sm.red2, sm.bmean, mxa, mya);
    if (tid < A) {
      rx = sm.ax[w][tid];
      ry = sm.ay[w][tid];
      px = (double)rx - mxa + xc;
      py = (double)ry - mya;
    }
  }
  // stash unsorted, then rank-sort by x: FP32 keys order the FP64 values
  // exactly except between equal keys, where the FP64 values decide
  const float pxf = (float)px;
  if (tid < A) { sm.X[w][tid] = px; sm.Y[w][tid] = py; sm.Xf[w][tid] = pxf; }
  else if (tid < ((A + 3) & ~3)) sm.Xf[w][tid] = INFINITY;   // keys past A: never below a key
  if (tid < kMaxA) sm.hits[w][tid] = 0;   // nucleons per rank (the pairing rewrites hits)
  __syncthreads();
  int rank = 0;
  if (tid < A) {
    for (int j = 0; j < A; j += 4) {
      const float4 k4 = *reinterpret_cast<const float4 *>(&sm.Xf[w][j]);
      rank += (k4.x < pxf) + (k4.y < pxf) + (k4.z < pxf) + (k4.w < pxf);
    }
    atomicAdd(&sm.hits[w][rank], 1);
  }
  __syncthreads();
  // nucleons with equal FP32 keys, and only those, share a rank (rare): the
  // FP64 values, then the index, decide between them
  const bool tie = tid < A && sm.hits[w][rank] > 1;
  if (__syncthreads_or(tie)) {
    if (tie) {
      for (int j = 0; j < A; j++) {
        if (sm.Xf[w][j] != pxf || j == tid) continue;
        const double xj = sm.X[w][j];
        rank += (xj < px) || (xj == px && j < tid);
      }
    }
    __syncthreads();
  }
  if (tid < A) {
    sm.X[w][rank] = px; sm.Y[w][rank] = py;
    sm.Xf[w][rank] = (float)px; sm.Yf[w][rank] = (float)py;
    if (!inj_xy) { sm.ax[w][rank] = rx; sm.ay[w][rank] = ry; }   // nucleus-frame positions, same order
    if (ntan)
      for (int c = 0; c < 4; c++) ntan[4 * rank + c] = (double)tg[c];
  }
  __syncthreads();
}

// Gamma(k, theta) weight of one source (slot) from the event's fluctuation
// stream: the method of Marsaglia and Tsang ("A simple method for
// generating gamma variables", ACM TOMS 26 (2000) 363) with
// Gamma(k) = Gamma(k+1) U^(1/k) for k < 1 and Box-Muller normals; iteration
// t draws counters 32 slot + 2t, 2t + 1 (t < 15), the k < 1 uniform counter
// 32 slot + 31.  The reference draws the same distribution from GSL
// (gsl_ran_gamma, src/MCnucl.cpp:1271-1301).
__device__ double gamma_weight(uint64_t seed, uint64_t ev, int attempt, uint32_t slot, double k, double theta) {
  return gamma_philox(seed, ev, stream_id(attempt, ST_FLUCT), 32 * slot, k, theta);
}

// tangent of nucleon k (sorted order, projectile first) of event e
__device__ __forceinline__ float4 nucleon_tangent(const double *ntan, int e, int AB, int k) {
  const double *t = ntan + ((size_t)e * AB + k) * 4;
  return make_float4((float)t[0], (float)t[1], (float)t[2], (float)t[3]);
}

// Bounding-box edges of a nucleon at x (Particle::Particle + calculateBounds,
// src/Particle.cpp:16-24,94-99, with all quarks at the nucleon centre).
__device__ __forceinline__ double box_lo(double x, const DevParams &P) {
  return x - 4 * fmax(P.width, P.quark_width);   // = min(x - 4w, x - 4 w_q), exactly
}
__device__ __forceinline__ double box_hi(double x, const DevParams &P) {
  return x + 4 * fmax(P.width, P.quark_width);
}

// signed-integer key with the order of the FP64 values
__device__ __forceinline__ long long order_key(double d) {
  long long b = __double_as_longlong(d);
  return b >= 0 ? b : b ^ 0x7fffffffffffffffLL;
}
__device__ __forceinline__ double from_order_key(long long k) {
  return __longlong_as_double(k >= 0 ? k : k ^ 0x7fffffffffffffffLL);
}

// Target range swept for projectile i by MCnucl::getBinaryCollision
// (src/MCnucl.cpp:244-292): from the first target whose box right edge
// reaches the projectile box's left edge, through the first target whose
// box left edge lies beyond the projectile box's right edge (the sweep
// tests that one too).  Both nuclei are sorted by x, so binary searches
// find both ends.
__device__ __forceinline__ void sweep_range(const SampleSmem &sm, const DevParams &P, int i, int B, int &lo,
                                            int &hi) {
  double pxl = box_lo(sm.X[0][i], P), pxr = box_hi(sm.X[0][i], P);
  int a = 0, b = B;
  while (a < b) {  // first j with box_hi(xj) >= pxl
    int m = (a + b) >> 1;
    if (box_hi(sm.X[1][m], P) >= pxl) b = m; else a = m + 1;
  }
  lo = a;
  int c = lo, d = B;
  while (c < d) {  // first j >= lo with box_lo(xj) > pxr
    int m = (c + d) >> 1;
    if (box_lo(sm.X[1][m], P) > pxr) d = m; else c = m + 1;
  }
  // inclusive; nothing is swept when the first candidate already lies
  // beyond the projectile box (the loop condition fails before any test)
  hi = (c == lo) ? lo - 1 : (c < B ? c : B - 1);
}

// Targets that can meet projectile i under the disk test: |x_j - x_i| <= rad
// (rad above the hit radius with margin); the targets are sorted by x, so
// two binary searches on the FP32 keys find the inclusive range [lo, hi].
// Pairs outside it fail the test, so the hits (and their order) are those
// of the full scan.
__device__ __forceinline__ void disk_range(const SampleSmem &sm, int i, int B, float rad, int &lo, int &hi) {
  const float xl = sm.Xf[0][i] - rad, xr = sm.Xf[0][i] + rad;
  int a = 0, b = B;
  while (a < b) {   // first j with x_j >= xl
    const int m = (a + b) >> 1;
    if (sm.Xf[1][m] >= xl) b = m; else a = m + 1;
  }
  int c = a, d = B;
  while (c < d) {   // first j with x_j > xr
    const int m = (c + d) >> 1;
    if (sm.Xf[1][m] > xr) d = m; else c = m + 1;
  }
  lo = a;
  hi = c - 1;
}

// MCnucl::hit (src/MCnucl.cpp:357-385) for projectile i, target j.  The disk
// test is decided in FP32 away from the threshold and in FP64, rounded as the
// reference rounds, near it.
__device__ __forceinline__ bool pair_hit(const SampleSmem &sm, const DevParams &P, int i, int j, float dsq_lo,
                                         float dsq_hi, uint64_t ev, int attempt, int B, bool swept) {
  float dx = sm.Xf[1][j] - sm.Xf[0][i], dy = sm.Yf[1][j] - sm.Yf[0][i];
  float d2 = dx * dx + dy * dy;
  if (swept) {
    // y-overlap of the bounding boxes (src/MCnucl.cpp:272-274)
    float ady = fabsf(dy), lim = sm.sc.box_lim;
    if (ady > lim * (1.f + 1e-5f)) return false;
    if (ady > lim * (1.f - 1e-5f)) {
      double yi = sm.Y[0][i], yj = sm.Y[1][j];
      if (!(box_lo(yi, P) <= box_hi(yj, P) && box_hi(yi, P) >= box_lo(yj, P))) return false;
    }
  }
  if (P.collision_criterion == 1) {
    if (d2 < dsq_lo) return true;
    if (d2 > dsq_hi) return false;
    double b = __dsqrt_rn(sq_dist_rn(sm.X[0][i], sm.Y[0][i], sm.X[1][j], sm.Y[1][j]));
    return __dmul_rn(b, b) <= P.dsq;
  }
  // Gaussian profile: P = 1 - exp(-sigma_gg exp(-b^2/4w^2)/(4 pi w^2))
  const float w2 = sm.sc.w2;
  if (d2 > 576.f * w2) return false;  // P < 1e-60 beyond 24 w
  float uf, unusedf;   // (float) of the FP64 uniform, without FP64 arithmetic
  uniform2f(P.seed, ev, stream_id(attempt, ST_COLL), (uint32_t)(i * B + j), uf, unusedf);
  float pf = 1.f - expf(-sm.sc.sigma_gg * expf(-d2 / (4.f * w2)) / (4.f * 3.14159265f * w2));
  if (uf < pf - 1e-5f) return true;
  if (uf > pf + 1e-5f) return false;
  double u, unused;
  uniform2(P.seed, ev, stream_id(attempt, ST_COLL), (uint32_t)(i * B + j), u, unused);
  double b = __dsqrt_rn(sq_dist_rn(sm.X[0][i], sm.Y[0][i], sm.X[1][j], sm.Y[1][j]));
  double w = P.width;
  return u < 1. - exp(-P.sigma_gg * exp(-b * b / (4. * w * w)) / (4. * M_PI * w * w));
}

// trunc_index(a + b, mn, d) with a + b rounded in FP64 as the reference
// rounds the edge, decided from the FP32 copies af, bf, mnf when they
// settle it: the FP32 value of t = (a + b - mn) / d is off by at most
// 3 2^-24 (|a| + |b| + |mn|) / d + 2^-23 |t| < 6e-4 while
// (|a| + |b| + |mn|) / d < 2000, so a fractional part 1e-3 away from an
// integer truncates as the exact value does.
__device__ __forceinline__ int edge_index(double a, double b, float af, float bf, double mn, float mnf, double d,
                                          float inv_d) {
  const float t = ((af + bf) - mnf) * inv_d;
  const float f = floorf(t), fr = t - f;
  if ((fabsf(af) + fabsf(bf) + fabsf(mnf)) * inv_d < 2000.f && fr > 1e-3f && fr < 1.f - 1e-3f) {
    const int i = (int)f;
    return (t < 0.f) ? i + 1 : i;   // truncation toward zero
  }
  return trunc_index(a + b, mn, d, inv_d);
}

// window [x - h, x + h) of a source at x (FP32 copy xf) on the grid axis
// starting at mn: the columns (rows) the reference's truncations give
__device__ __forceinline__ void set_window_c(Source &s, double x, float xf, double h, float hf, double mn,
                                             float mnf, double d, float inv_d, int nmax, bool is_x) {
  int l = edge_index(x, -h, xf, -hf, mn, mnf, d, inv_d), r = edge_index(x, h, xf, hf, mn, mnf, d, inv_d);
  l = max(0, l);
  r = min(nmax, r);
  if (is_x) { s.xl = (int16_t)l; s.xr = (int16_t)r; }
  else { s.yl = (int16_t)l; s.yr = (int16_t)r; }
}

// ----------------------------------------------------------------- kernel
// systems / ev_sys (mixed batches, else NULL): the system parameters of
// event e are systems[ev_sys[e]]; order (else NULL): the order in which the
// CTAs take the events (heavy systems first).
// six CTAs per SM (shared memory allows six; more resident warps beat the spills
// this register budget costs)
__global__ void __launch_bounds__(kNT, 6) k_sample_pair(DevParams P_in, uint64_t first_event, int n_events,
                                                     const double *inj_proj, const double *inj_targ,
                                                     const double *inj_b, EventRec *recs, Source *srcs,
                                                     double *out_pos, uint8_t *out_wounded,
                                                     const SystemDev *systems, const int *ev_sys,
                                                     const int *order, TangentIO tio, const uint64_t *ev_base,
                                                     int *ticket) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SampleSmem &sm = *reinterpret_cast<SampleSmem *>(smem_raw);
  __shared__ DevParams s_P;   // the context's parameters with the event's system
  const DevParams &P = s_P;
  const int tid = threadIdx.x;
  const bool inject = inj_proj != nullptr;
  const float inv_dx = (float)(1.0 / P_in.dx), inv_dy = (float)(1.0 / P_in.dy);

  // events by ticket (retries make their costs uneven), in `order` when given
  const EventQueue q{order, ticket};
  __shared__ int s_k;
  for (int k_ev = queue_first(q, &s_k); k_ev < n_events; k_ev = queue_next(q, k_ev, &s_k)) {
    const int e = queue_event(q, k_ev);
    __syncthreads();   // s_P of the previous event is no longer read
    if (tid == 0) {
      s_P = P_in;
      if (systems) {
        const SystemDev &sd = systems[ev_sys[e]];
        s_P.nuc[0] = sd.nuc[0];
        s_P.nuc[1] = sd.nuc[1];
        s_P.dsq = sd.dsq;
        s_P.sigma_gg = sd.sigma_gg;
        s_P.sigin = sd.sigin;
        s_P.bmin = sd.bmin;
        s_P.bmax = sd.bmax;
        s_P.npmin = sd.npmin;
        s_P.npmax = sd.npmax;
      }
      for (int w = 0; w < 2; w++) {
        NucleusDev &nu = s_P.nuc[w];
        nu.R_f = (float)nu.R;
        nu.a_f = (float)nu.a;
        nu.rmax_f = (float)nu.rmax_cut;
        nu.rw_max_f = (float)nu.rw_max;
        nu.beta2_f = (float)nu.beta2;
        nu.beta4_f = (float)nu.beta4;
        nu.dmin2_f = (float)(nu.d_min * nu.d_min);
        nu.nslab = nu.d_min > 0 ? max(1, min(kSlab, (int)floorf(2.f * nu.rmax_f / (1.01f * (float)nu.d_min)))) : 1;
        nu.slab_inv_w = (float)nu.nslab / (2.f * nu.rmax_f);
      }
      SampleConsts &c = sm.sc;
      c.cbox = 4 * fmax(s_P.width, s_P.quark_width);
      c.d_max = s_P.shape_of_nucleons == 1 ? 2. * sqrt(s_P.dsq) : 5. * s_P.width;
      c.disk_val_d = 10.0 / s_P.sigin;
      c.cbox_f = (float)c.cbox;
      c.d_max_f = (float)c.d_max;
      c.xmin_f = (float)s_P.xmin;
      c.ymin_f = (float)s_P.ymin;
      c.dsq_lo = (float)s_P.dsq * (1.f - 1e-4f);
      c.dsq_hi = (float)s_P.dsq * (1.f + 1e-4f);
      c.hit_rad = sqrtf(c.dsq_hi) * (1.f + 1e-4f);   // |dx| beyond it: no disk hit
      c.peak = (float)s_P.peak;
      c.disk_val = (float)c.disk_val_d;
      c.wn = (float)((1.0 - s_P.alpha) / 2.);
      c.box_lim = 4.f * (float)(fmax(s_P.width, s_P.quark_width)) * 2.f;
      c.w2 = (float)s_P.w2;
      c.sigma_gg = (float)s_P.sigma_gg;
      // The reference only tests pairs its box sweep reaches.  For the disk test
      // with a hit radius well inside the box width every hit pair is swept, so
      // all pairs are tested; otherwise the sweep's tested set is reproduced.
      c.swept = s_P.collision_criterion != 1 || sqrt(s_P.dsq) > 7.9 * fmax(s_P.width, s_P.quark_width);
    }
    __syncthreads();
    const int A = P.nuc[0].A, B = P.nuc[1].A;
    const float dsq_lo = sm.sc.dsq_lo, dsq_hi = sm.sc.dsq_hi, hit_rad = sm.sc.hit_rad;
    const bool swept = sm.sc.swept;
    const uint64_t ev = (ev_base ? *ev_base : 0) + first_event + (uint64_t)e;
    int status = 0, attempt = 0, ncoll = 0, np1 = 0, np2 = 0;
    for (;; attempt++) {
      if (attempt >= P.max_attempts) { status = 3; break; }
      // impact parameter (MakeDensity.cpp:2149)
      if (tid == 0) {
        // a given impact parameter (injected nuclei, or nuclei drawn at a
        // given b: MCnucl::generateNuclei(b)), else drawn
        if (inj_b) sm.b = inj_b[e];
        else if (inject) sm.b = 0.0;
        if (!inject) {
          if (!inj_b) {
            double u, unused;
            uniform2(P.seed, ev, stream_id(attempt, ST_EVENT), 0, u, unused);
            sm.b = sqrt((P.bmax * P.bmax - P.bmin * P.bmin) * u + P.bmin * P.bmin);
          }
          // nucleus orientations (cos theta, phi)
          for (int w = 0; w < 2; w++) {
            double o0, o1;
            uniform2(P.seed, ev, stream_id(attempt, ST_EVENT), 1 + w, o0, o1);
            sm.ori[w][0] = 1.0 - 2.0 * o0;
            sm.ori[w][1] = 2 * M_PI * o1;
            // a table nucleus's configuration (the reference: rand() % nconf)
            if (P.nuc[w].conf) {
              uniform2(P.seed, ev, stream_id(attempt, ST_CONF), (uint32_t)w, o0, o1);
              sm.cfg_idx[w] = min((int)(o0 * P.nuc[w].nconf), P.nuc[w].nconf - 1);
            }
          }
        }
      }
      __syncthreads();
      const double b = sm.b;
      bool ok = true;
      // the nuclei in their own frames: two large Woods-Saxon nuclei at
      // once, one per half of the CTA (each half's barriers its own);
      // otherwise one after the other by the whole CTA (a nucleus of up to
      // ~100 nucleons takes about as many half-size batches as full ones, and
      // measured slower).  The streams are per nucleus, so the order does not
      // change them.
      if (!inject && P.nuc[0].A > 100 && P.nuc[1].A > 100 && !P.nuc[0].conf && !P.nuc[1].conf) {
        const int h = tid / (kNT / 2);
        const bool okh = sample_ws<kNT / 2>(sm, sm.samp.half[h], P.nuc[h], h, P.seed, ev, attempt,
                                            (float)sm.ori[h][0], (float)sm.ori[h][1], HalfSync{h});
        ok = __syncthreads_and(okh) && ok;
      } else if (!inject) {
        for (int w = 0; w < 2; w++) {
          const NucleusDev &nu = P.nuc[w];
          // rounded to float for the FP32 samplers
          const float ctr = (float)sm.ori[w][0], phir = (float)sm.ori[w][1];
          if (nu.conf) {
            // placed from the table below
          } else if (nu.A == 1) {
            if (tid == 0) { sm.ax[w][0] = 0.f; sm.ay[w][0] = 0.f; sm.az[w][0] = 0.f; }
            __syncthreads();
          } else if (nu.A == 2) {
            if (tid == 0) {
              double u, unused;
              uniform2(P.seed, ev, stream_id(attempt, ST_DEUT), (uint32_t)w, u, unused);
              double d = hulthen_inv(u);
              float x1 = (float)(d / 2.0), y1 = 0.f, z1 = 0.f;
              rotate3f(x1, y1, z1, ctr, phir);
              sm.ax[w][0] = x1; sm.ay[w][0] = y1; sm.az[w][0] = z1;
              sm.ax[w][1] = -x1; sm.ay[w][1] = -y1; sm.az[w][1] = -z1;
            }
            __syncthreads();
          } else {
            ok = ok && sample_ws<kNT>(sm, sm.samp.full, nu, w, P.seed, ev, attempt, ctr, phir, FullSync{});
          }
        }
      }
      for (int w = 0; w < 2; w++) {
        const NucleusDev &nu = P.nuc[w];
        const double xc = (w == 0 ? b : -b) / 2.0;
        double *ntan = tio.ntan ? tio.ntan + ((size_t)e * (A + B) + (w == 0 ? 0 : A)) * 4 : nullptr;
        if (inject) {
          const double *itan = w == 0 ? tio.inj_proj : tio.inj_targ;
          place_sorted(sm, w, nu.A, 0.0, (w == 0 ? inj_proj : inj_targ) + (size_t)e * 2 * nu.A, nu,
                       itan ? itan + (size_t)e * 4 * nu.A : nullptr, ntan);
          continue;
        }
        const double *cfg = nu.conf ? nu.conf + (size_t)sm.cfg_idx[w] * 3 * nu.A : nullptr;
        place_sorted(sm, w, nu.A, xc, nullptr, nu, nullptr, ntan, cfg, sm.ori[w][0], sm.ori[w][1]);
      }
      if (!ok) { status = 3; break; }
      // ---- pairing: thread i tests projectile i against every target
      if (tid < B) sm.hits[1][tid] = 0;
      __syncthreads();
      int cnt = 0;
      if (tid < A) {
        int jlo = 0, jhi = B - 1;
        if (swept) sweep_range(sm, P, tid, B, jlo, jhi);
        else if (P.collision_criterion == 1) disk_range(sm, tid, B, hit_rad, jlo, jhi);
        for (int j = jlo; j <= jhi; j++) {
          if (pair_hit(sm, P, tid, j, dsq_lo, dsq_hi, ev, attempt, B, swept)) {
            cnt++;
            atomicAdd(&sm.hits[1][j], 1);
          }
        }
        sm.hits[0][tid] = cnt;
      }
      __syncthreads();
      block_sum3_i(tid < A && sm.hits[0][tid] > 0, tid < B && sm.hits[1][tid] > 0, cnt, sm.ired, np1, np2, ncoll);
      __syncthreads();
      if (inject) break;
      int np = np1 + np2;
      if (ncoll > 0 && np >= P.npmin && np <= P.npmax) break;   // CentralityCut
    }

    // ---- outputs: positions, wounded flags
    const int AB = A + B;
    if (out_pos) {
      for (int k = tid; k < AB; k += kNT) {
        int w = k < A ? 0 : 1, i = k < A ? k : k - A;
        out_pos[((size_t)e * AB + k) * 2] = sm.X[w][i];
        out_pos[((size_t)e * AB + k) * 2 + 1] = sm.Y[w][i];
      }
    }
    if (out_wounded) {
      for (int k = tid; k < AB; k += kNT) {
        int w = k < A ? 0 : 1, i = k < A ? k : k - A;
        out_wounded[(size_t)e * AB + k] = sm.hits[w][i] > 0;
      }
    }

    // ---- splat sources (with their position tangents when requested)
    Source *S = srcs + (size_t)e * P.max_src;
    float4 *stan = tio.stan ? tio.stan + (size_t)e * P.max_src : nullptr;
    const double d_max = sm.sc.d_max;
    const float d_max_f = sm.sc.d_max_f, xmin_f = sm.sc.xmin_f, ymin_f = sm.sc.ymin_f;
    const int model = P.which_mc_model;
    const bool box_src = (model == 5 && P.sub_model == 1) || model == 7;
    const bool coll_src = model == 5 && P.alpha > 1e-8;
    const bool coll_rec = coll_src || P.want_binary;   // density sources, or records for rho_binary
    const bool thick_src = model == 1 || P.want_ta || P.want_tb;
    const bool disk_n = P.shape_of_nucleons == 1, disk_e = P.shape_of_entropy == 1;
    const float peak = sm.sc.peak;
    const float disk_val = sm.sc.disk_val;

    // region of the eccentricity mask: union of participant boxes and the
    // (unset, all-zero) collision boxes.  Box edges are x -+ c with
    // c = 4 max(w, quark_width), monotone in x, so the region follows from
    // the extreme participant coordinates, found with integer order keys
    // of the FP64 values; thread 0 then derives the region (FP64).
    const double cbox = sm.sc.cbox;
    const float cbox_f = sm.sc.cbox_f;
    {
      long long kx0 = LLONG_MAX, kx1 = LLONG_MIN, ky0 = LLONG_MAX, ky1 = LLONG_MIN;
      for (int k = tid; k < AB; k += kNT) {
        int w = k < A ? 0 : 1, i = k < A ? k : k - A;
        if (sm.hits[w][i] == 0) continue;
        long long kx = order_key(sm.X[w][i]), ky = order_key(sm.Y[w][i]);
        kx0 = min(kx0, kx); kx1 = max(kx1, kx); ky0 = min(ky0, ky); ky1 = max(ky1, ky);
      }
      for (int o = 16; o; o >>= 1) {
        kx0 = min(kx0, __shfl_xor_sync(0xffffffffu, kx0, o));
        kx1 = max(kx1, __shfl_xor_sync(0xffffffffu, kx1, o));
        ky0 = min(ky0, __shfl_xor_sync(0xffffffffu, ky0, o));
        ky1 = max(ky1, __shfl_xor_sync(0xffffffffu, ky1, o));
      }
      __syncthreads();
      if ((tid & 31) == 0) {
        int w = tid >> 5;
        sm.lred[w] = kx0; sm.lred[8 + w] = kx1; sm.lred[16 + w] = ky0; sm.lred[24 + w] = ky1;
      }
      __syncthreads();
      if (tid == 0) {
        for (int q = 0; q < kNT / 32; q++) {
          kx0 = min(kx0, sm.lred[q]); kx1 = max(kx1, sm.lred[8 + q]);
          ky0 = min(ky0, sm.lred[16 + q]); ky1 = max(ky1, sm.lred[24 + q]);
        }
        double rxl, rxr, ryl, ryr;
        if (np1 + np2 == 0) {
          rxl = rxr = ryl = ryr = 0.0;
        } else {
          rxl = from_order_key(kx0) - cbox; rxr = from_order_key(kx1) + cbox;
          ryl = from_order_key(ky0) - cbox; ryr = from_order_key(ky1) + cbox;
          if (ncoll > 0) {
            rxl = fmin(rxl, 0.0); rxr = fmax(rxr, 0.0); ryl = fmin(ryl, 0.0); ryr = fmax(ryr, 0.0);
          }
        }
        SampleConsts &c = sm.sc;
        c.rxl = rxl; c.ryl = ryl;
        c.rxl_f = (float)rxl; c.ryl_f = (float)ryl;
        c.nXp = (int)((rxr - rxl) / P.dx); c.nYp = (int)((ryr - ryl) / P.dy);
        c.ioff = (int)((rxl - P.xmin) / P.dx); c.joff = (int)((ryl - P.ymin) / P.dy);
      }
      __syncthreads();
    }
    const double rxl = sm.sc.rxl, ryl = sm.sc.ryl;
    const float rxl_f = sm.sc.rxl_f, ryl_f = sm.sc.ryl_f;
    const int nXp = sm.sc.nXp, nYp = sm.sc.nYp, ioff = sm.sc.ioff, joff = sm.sc.joff;

    // Records of the event: [participant boxes, when they splat][thickness
    // records][collisions][participant boxes, mask-only][spectators].  The
    // splat sources lead (nsplat of them); each kind is in the reference's
    // order (participants: nucleon order, projectile then target).
    const int Np = np1 + np2;
    const int ncs = (coll_rec && ncoll > 0) ? min(ncoll, P.max_coll) : 0;
    const int thick_base = box_src ? Np : 0;
    const int coll_base = thick_base + (thick_src ? Np : 0);
    const int mask_base = coll_base + ncs;
    const int nsplat = coll_base + (coll_src ? ncs : 0);
    int nsrc = mask_base + (box_src ? 0 : Np);
    int imin = P.nx, imax = 0, jmin = P.ny, jmax = 0;
    {
      // one box record per participant (a splat source, or mask-only when the
      // model does not splat boxes) plus a thickness record when T_A/T_B are made
      int pdone = 0;   // participants placed
      // prefix over wounded flags
      int flag = 0;
      for (int k = tid; k < ((AB + kNT - 1) / kNT) * kNT; k += kNT) {
        int w = k < A ? 0 : 1, i = k < A ? k : k - A;
        flag = (k < AB) && sm.hits[w][i] > 0;
        // block exclusive scan of flag
        int v = flag;
        for (int o = 1; o < 32; o <<= 1) {
          int t = __shfl_up_sync(0xffffffffu, v, o);
          if ((tid & 31) >= o) v += t;
        }
        if ((tid & 31) == 31) sm.ired[tid >> 5] = v;
        __syncthreads();
        int woff = 0, tot = 0;
        for (int q = 0; q < kNT / 32; q++) {
          if (q < (tid >> 5)) woff += sm.ired[q];
          tot += sm.ired[q];
        }
        const int p = pdone + woff + v - flag;   // participant index
        if (flag) {
          const double x = sm.X[w][i], y = sm.Y[w][i];
          const float xf = sm.Xf[w][i], yf = sm.Yf[w][i];
          {
            Source s;
            s.x = x; s.y = y;
            if (box_src) {
              set_window_c(s, x, xf, cbox, cbox_f, P.xmin, xmin_f, P.dx, inv_dx, P.nx, true);
              set_window_c(s, y, yf, cbox, cbox_f, P.ymin, ymin_f, P.dy, inv_dy, P.ny, false);
            } else {
              s.xl = s.xr = s.yl = s.yr = 0;   // eccentricity mask only
            }
            // mask lattice of MakeDensity.cpp:2356-2358 (its y upper bound divides by dx)
            int x0 = edge_index(x, -cbox, xf, -cbox_f, rxl, rxl_f, P.dx, inv_dx);
            int x1 = edge_index(x, cbox, xf, cbox_f, rxl, rxl_f, P.dx, inv_dx);
            int y0 = edge_index(y, -cbox, yf, -cbox_f, ryl, ryl_f, P.dy, inv_dy);
            int y1 = edge_index(y, cbox, yf, cbox_f, ryl, ryl_f, P.dx, inv_dx);
            s.mx0 = (int16_t)(max(0, x0) + ioff); s.mx1 = (int16_t)(min(nXp, x1) + ioff);
            s.my0 = (int16_t)(max(0, y0) + joff); s.my1 = (int16_t)(min(nYp, y1) + joff);
            s.kind = box_src ? (SRC_PART_BOX | (disk_e ? 16 : 0)) : 3;
            s.plane = (model == 7 && w == 1) ? 1 : 0;
            s.weight = disk_e ? disk_val * (model == 5 ? sm.sc.wn : 1.f) : peak * (model == 5 ? sm.sc.wn : 1.f);
            // Particle::getSmoothDensity's multiplicity factor (MCnucl::selectFluctFactors)
            if (P.fluct)
              s.weight = (float)((double)s.weight *
                                 gamma_weight(P.seed, ev, attempt, (uint32_t)k, P.fluct_k_part, P.fluct_th_part));
            // a Woods-Saxon nucleon is constructed at its nucleus-frame
            // position and then moved (Nucleus::populate,
            // src/Nucleus.cpp:274-309, Particle::setX/setY): its base box
            // stays there, and the averaged mode's rotation brings it back;
            // light nuclei are constructed in place (:199-236)
            if (!inject && (w == 0 ? A : B) > 2 && !P.nuc[w].conf) {
              s.kind |= SRC_RAW_BASE;
              s.bx = sm.ax[w][i];
              s.by = sm.ay[w][i];
            } else {
              s.bx = s.by = 0.f;
            }
            const int pos = box_src ? p : mask_base + p;
            if (stan) stan[pos] = nucleon_tangent(tio.ntan, e, AB, k);
            set_grid_offsets(s, P);
            S[pos] = s;
          }
          if (thick_src) {
            Source s;
            s.x = x; s.y = y;
            set_window_c(s, x, xf, d_max, d_max_f, P.xmin, xmin_f, P.dx, inv_dx, P.nx, true);
            set_window_c(s, y, yf, d_max, d_max_f, P.ymin, ymin_f, P.dy, inv_dy, P.ny, false);
            s.mx0 = s.mx1 = s.my0 = s.my1 = 0;
            s.kind = SRC_THICK | (disk_n ? 16 : 0);
            s.plane = model == 1 ? w : 1 + w;   // MC-KLN splats T_A, T_B only
            s.weight = disk_n ? disk_val : peak;
            s.bx = s.by = 0.f;
            if (stan) stan[thick_base + p] = nucleon_tangent(tio.ntan, e, AB, k);
            set_grid_offsets(s, P);
            S[thick_base + p] = s;
          }
        }
        pdone += tot;
        __syncthreads();
      }
    }
    // collision sources, ordered by (projectile, target) index
    if (coll_rec && ncoll > 0) {
      // exclusive scan of per-projectile hit counts
      int c = tid < A ? sm.hits[0][tid] : 0;
      int v = c;
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if ((tid & 31) >= o) v += t;
      }
      if ((tid & 31) == 31) sm.ired[tid >> 5] = v;
      __syncthreads();
      int woff = 0;
      for (int q = 0; q < (tid >> 5); q++) woff += sm.ired[q];
      __syncthreads();
      int pos = woff + v - c;
      if (ncoll > P.max_coll) status = 6;
      if (tid < A && c > 0) {
        int jlo = 0, jhi = B - 1;
        if (swept) sweep_range(sm, P, tid, B, jlo, jhi);
        else if (P.collision_criterion == 1) disk_range(sm, tid, B, hit_rad, jlo, jhi);
        for (int j = jlo; j <= jhi && pos < ncs; j++) {
          if (!pair_hit(sm, P, tid, j, dsq_lo, dsq_hi, ev, attempt, B, swept)) continue;
          Source s;
          s.x = (sm.X[0][tid] + sm.X[1][j]) / 2.0;
          s.y = (sm.Y[0][tid] + sm.Y[1][j]) / 2.0;
          set_window_c(s, s.x, (float)s.x, d_max, d_max_f, P.xmin, xmin_f, P.dx, inv_dx, P.nx, true);
          set_window_c(s, s.y, (float)s.y, d_max, d_max_f, P.ymin, ymin_f, P.dy, inv_dy, P.ny, false);
          s.mx0 = s.mx1 = s.my0 = s.my1 = 0;
          s.plane = 0;
          double aw = 0.;
          if (model == 5 && P.sub_model == 2) aw = (double)(1 / c) + (double)(1 / sm.hits[1][j]);
          s.kind = coll_src ? (SRC_COLL | (disk_e ? 16 : 0) | ((int)aw << SRC_AW_SHIFT)) : SRC_BINARY;
          double fw = P.alpha + (1. - P.alpha) * aw;
          // CollisionPair::getfluctfactor (src/MCnucl.cpp:730-731)
          if (P.fluct)
            fw *= gamma_weight(P.seed, ev, attempt, (uint32_t)(AB + tid * B + j), P.fluct_k_coll, P.fluct_th_coll);
          s.weight = (float)((disk_e ? sm.sc.disk_val_d : P.peak) * fw);
          s.bx = s.by = 0.f;
          if (stan) {
            const float4 ta = nucleon_tangent(tio.ntan, e, AB, tid), tb = nucleon_tangent(tio.ntan, e, AB, A + j);
            stan[coll_base + pos] = make_float4(0.5f * (ta.x + tb.x), 0.5f * (ta.y + tb.y), 0.5f * (ta.z + tb.z),
                                           0.5f * (ta.w + tb.w));
          }
          set_grid_offsets(s, P);
          S[coll_base + pos] = s;
          pos++;
        }
      }
    }
    __syncthreads();
    // spectators (MCnucl::getSpectators, src/MCnucl.cpp:1223-1248): the
    // nucleons without a collision, projectile then target, nucleon order
    if (P.want_spect) {
      for (int k0 = 0; k0 < AB; k0 += kNT) {
        const int k = k0 + tid, w = k < A ? 0 : 1, i = k < A ? k : k - A;
        const bool flag = k < AB && sm.hits[w][i] == 0;
        const unsigned bal = __ballot_sync(0xffffffffu, flag);
        __syncthreads();
        if ((tid & 31) == 0) sm.ired[tid >> 5] = __popc(bal);
        __syncthreads();
        int woff = 0, tot = 0;
        for (int q = 0; q < kNT / 32; q++) {
          woff += q < (tid >> 5) ? sm.ired[q] : 0;
          tot += sm.ired[q];
        }
        if (flag) {
          Source s;
          s.x = sm.X[w][i];
          s.y = sm.Y[w][i];
          set_window_c(s, s.x, sm.Xf[w][i], d_max, d_max_f, P.xmin, xmin_f, P.dx, inv_dx, P.nx, true);
          set_window_c(s, s.y, sm.Yf[w][i], d_max, d_max_f, P.ymin, ymin_f, P.dy, inv_dy, P.ny, false);
          s.mx0 = s.mx1 = s.my0 = s.my1 = 0;
          s.kind = SRC_SPECT | (disk_n ? 16 : 0);
          s.plane = w;
          s.weight = disk_n ? disk_val : peak;
          s.bx = s.by = 0.f;
          set_grid_offsets(s, P);
          S[nsrc + woff + __popc(bal & ((1u << (tid & 31)) - 1u))] = s;
        }
        nsrc += tot;
      }
      __syncthreads();
    }
    // bounding box of the splat windows (the density is zero outside them;
    // the records after the splat sources -- mask-only participant boxes,
    // collisions kept for other views, spectators -- do not widen it)
    for (int k = tid; k < nsplat; k += kNT) {
      Source s = S[k];
      if (s.xr > s.xl && s.yr > s.yl) {
        imin = min(imin, (int)s.xl); imax = max(imax, (int)s.xr);
        jmin = min(jmin, (int)s.yl); jmax = max(jmax, (int)s.yr);
      }
    }
    for (int o = 16; o; o >>= 1) {
      imin = min(imin, __shfl_xor_sync(0xffffffffu, imin, o));
      imax = max(imax, __shfl_xor_sync(0xffffffffu, imax, o));
      jmin = min(jmin, __shfl_xor_sync(0xffffffffu, jmin, o));
      jmax = max(jmax, __shfl_xor_sync(0xffffffffu, jmax, o));
    }
    if ((tid & 31) == 0) {
      int w = tid >> 5;
      sm.scan[w] = imin; sm.scan[8 + w] = imax; sm.scan[16 + w] = jmin; sm.scan[24 + w] = jmax;
    }
    __syncthreads();
    if (tid == 0) {
      for (int q = 0; q < kNT / 32; q++) {
        imin = min(imin, sm.scan[q]); imax = max(imax, sm.scan[8 + q]);
        jmin = min(jmin, sm.scan[16 + q]); jmax = max(jmax, sm.scan[24 + q]);
      }
      EventRec r;
      r.b = sm.b;
      r.npart1 = np1; r.npart2 = np2; r.ncoll = ncoll; r.nsrc = nsrc; r.nsplat = nsplat;
      r.attempts = attempt + 1; r.status = status;
      r.imin = imin; r.imax = imax; r.jmin = jmin; r.jmax = jmax;
      r.ev = ev;
      recs[e] = r;
      // Nucleus::populate's (cx, phi) of both nuclei (src/Nucleus.cpp:192-196),
      // in FP64 from the attempt's uniforms; zero for injected nuclei
      if (tio.orient) {
        double o[4] = {0.0, 0.0, 0.0, 0.0};
        if (!inject && status == 0) {
          for (int w = 0; w < 2; w++) {
            double o0, o1;
            uniform2(P.seed, ev, stream_id(attempt, ST_EVENT), 1 + w, o0, o1);
            o[2 * w] = 1.0 - 2.0 * o0;
            o[2 * w + 1] = 2 * M_PI * o1;
          }
        }
        for (int k = 0; k < 4; k++) tio.orient[4 * (size_t)e + k] = o[k];
      }
    }
    __syncthreads();
  }
}

size_t sample_pair_smem() { return sizeof(SampleSmem); }

cudaError_t launch_sample_pair(const DevParams &P, uint64_t first_event, int n_events, const double *inj_proj,
                               const double *inj_targ, const double *inj_b, EventRec *recs, Source *srcs,
                               double *out_pos, uint8_t *out_wounded, int grid, cudaStream_t st) {
  return launch_sample_pair_mixed(P, first_event, n_events, inj_proj, inj_targ, inj_b, recs, srcs, out_pos,
                                  out_wounded, nullptr, nullptr, nullptr, grid, st);
}

cudaError_t launch_sample_pair_mixed(const DevParams &P, uint64_t first_event, int n_events, const double *inj_proj,
                                     const double *inj_targ, const double *inj_b, EventRec *recs, Source *srcs,
                                     double *out_pos, uint8_t *out_wounded, const SystemDev *systems,
                                     const int *ev_sys, const int *order, int grid, cudaStream_t st,
                                     const TangentIO *tio, const uint64_t *ev_base, int *ticket) {
  size_t smem = sizeof(SampleSmem);
  // per launch: the attribute belongs to the current device's context
  cudaError_t ea = cudaFuncSetAttribute(k_sample_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (ea != cudaSuccess) return ea;
  if (ticket) {
    cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
  }
  k_sample_pair<<<grid, kNT, smem, st>>>(P, first_event, n_events, inj_proj, inj_targ, inj_b, recs, srcs, out_pos,
                                         out_wounded, systems, ev_sys, order, tio ? *tio : TangentIO{}, ev_base,
                                         ticket);
  return cudaGetLastError();
}

}  // namespace smc
