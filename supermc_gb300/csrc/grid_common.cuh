// Device helpers shared by the two grid kernels (the CUDA-core splat in
// k_grid.cu and the tensor-core contraction in k_grid_tc.cu): double-float
// reductions, the reference's exact per-cell inclusion rules, the six-point
// table interpolation and the eccentricity moments.
//
//   per-cell cuts       src/Particle.cpp:122-132, src/MCnucl.cpp:732-756
//   six-point lookup    src/arsenal.cpp:33-54 (used at src/MCnucl.cpp:654-687)
//   eps_n, <r^n>        src/MakeDensity.cpp:2244-2511, hot-spot mask src/MCnucl.cpp:1303-1323
#pragma once
#include <climits>

#include "smc_device.cuh"

namespace smc {

struct GroupSrc {
  double x, y;
  float xf, yf, weight;
  float gi0;               // x = xmin + (gi0 + gfx) dx: grid cell and fraction in [0, 1)
                           // (Source::gi0 .. gfy)
  float gfy, gj0;          // the same along y (8-byte aligned: read together by the
                           // accumulating lanes)
  float gfx;
  int16_t kind, plane;
  int16_t xl, xr, yl, yr;
};
static_assert(offsetof(GroupSrc, gfy) % 8 == 0, "column offsets read as one 8-byte word");

// 2^a (PTX ex2.approx.ftz.f32, relative error below 2^-22)
__device__ __forceinline__ float ex2f(float a) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}

// exp(-d^2 / 2w^2) of a grid distance d = (k - cell) - frac in grid units:
// 2^(-d^2 c) with c = spacing^2 log2(e) / (2 w^2)
__device__ __forceinline__ float gauss_grid(float k, float cell, float frac, float c) {
  const float d = (k - cell) - frac;
  return ex2f(-(d * d) * c);
}

// ---------------------------------------------------- double-float sums
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);   // TwoSum error
  e += a.lo + b.lo;
  float h = s + e;
  return {h, e - (h - s)};
}
__device__ __forceinline__ DF df_warp_sum(DF v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    DF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, w);
  }
  return v;
}
// Kahan-compensated FP32 accumulator
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ DF df() const { return {s, -c}; }
};

// Relative half width of the band around a cut dc <= rho2 inside which the
// FP32 distance does not decide a cell (the FP64 test does).  The FP32 grid
// coordinates and source positions that reach a cell are at most
// M = (grid extent) + rho in magnitude and each off by 2^-24 M, so
// |dc_FP32 - dc| <= 7.2e-7 rho M + 2.4e-7 rho^2; the band is three times
// that relative to rho^2, never wider than 1e-4.
__device__ __forceinline__ float cut_band(const DevParams &P, double rho2) {
  const double rho = sqrt(rho2);
  const double ext = fmax(fmax(fabs(P.xmin), fabs(P.xmin + (P.nx - 1) * P.dx)),
                          fmax(fabs(P.ymin), fabs(P.ymin + (P.ny - 1) * P.dy)));
  return rho > 0 ? (float)fmin(1e-4, 2.2e-6 * (ext + rho) / rho + 7.2e-7) : 1e-4f;
}

// exact per-cell inclusion, FP64 as the reference evaluates it
static __device__ __noinline__ bool cell_in_exact(const DevParams &P, double sx, double sy, int kind, int i, int j) {
  double xg = __dadd_rn(P.xmin, __dmul_rn((double)i, P.dx));
  double yg = __dadd_rn(P.ymin, __dmul_rn((double)j, P.dy));
  double dc = sq_dist_rn(sx, sy, xg, yg);
  if (kind & 16) return !(dc > P.dsq);                        // disk nucleons / entropy
  if ((kind & 15) == SRC_COLL) return dc <= __dmul_rn(25., P.w2);  // MCnucl.cpp:754
  double r = __dsqrt_rn(dc);                                  // Particle::getSmoothTn
  return !(r > __dmul_rn(5., P.width));
}

__device__ __forceinline__ float six_point(float x, float y, float v00, float v01, float v02, float v10, float v11,
                                           float v20) {
  float axx = 0.5f * (v00 - 2.f * v10 + v20);
  float axy = v00 - v01 - v10 + v11;
  float ayy = 0.5f * (v00 - 2.f * v01 + v02);
  float bx = 0.5f * (-3.f * v00 + 4.f * v10 - v20);
  float by = 0.5f * (-3.f * v00 + 4.f * v01 - v02);
  return axx * x * x + axy * x * y + ayy * y * y + bx * x + by * y + v00;
}

// Per-cell results of post_cell
enum CellCode : int {
  CELL_OK = 0,
  CELL_TABLE = 1,       // MC-KLN thickness beyond the dN/dy table (status 4)
  CELL_UNDECIDED = 8,   // MC-KLN: the FP32 thickness leaves the table cell
                        // floor(T/dT) undecided; it is decided from FP64 sums
                        // of the planes flagged below
  CELL_NEED_A = 16, CELL_NEED_B = 32
};

// The six-point interpolation of the dN/dy table in table cell (ii, jj) at
// offsets (fi, fj) in lattice units (src/MCnucl.cpp:672-676)
// (sixPoint2dInterp, src/arsenal.cpp:33-54, with the cell's coefficients
// taken in FP64 from the table once per context: two 16-byte loads and five
// FMAs per cell)
__device__ __forceinline__ float kln_interp(const DevParams &P, int ii, int jj, float fi, float fj) {
  const float4 *c = P.kln_coef + 2 * ((size_t)ii * P.kln_tmax + jj);
  const float4 a = __ldg(c), b = __ldg(c + 1);   // axx, axy, ayy, bx | by, v00
  return fmaf(fmaf(a.x, fi, fmaf(a.y, fj, a.w)), fi, fmaf(fmaf(a.z, fj, b.x), fj, b.y));
}

// Relative error bound of an event's FP32 thickness sums: the per-term
// bound P.kln_band plus one rounding (2^-24) per added term, at most
// max(Npart1, Npart2) terms.
__device__ __forceinline__ float kln_event_band(const DevParams &P, const EventRec &rec) {
  return fmaf((float)max(rec.npart1, rec.npart2), 5.9604645e-8f, P.kln_band);
}

// Per-cell post-op of the splat planes a0..a2 (np planes): the density v and
// the thickness outputs t1, t2 (MCnucl::setDensity, src/MCnucl.cpp:654-811).
//   model 5 (Glauber): v = a0; planes 1, 2 are T_A, T_B when requested
//   model 7: v = sqrt(T_A T_B)
//   model 1 (MC-KLN): planes are T_A, T_B; v = dN/dy from the six-point
//     interpolation in the table at di = T_A/dT, dj = T_B/dT, table cell
//     (floor di, floor dj); CELL_TABLE when the thickness lies beyond the
//     table (the reference exits there, src/MCnucl.cpp:665-670).  The FP32
//     thickness is within a relative `band` of the reference's FP64 sum;
//     when di or dj is that close to an integer the table cell (or, for a
//     cell with a zero thickness, whose value is 0 in any table cell, the
//     bound test) is undecided in FP32: CELL_UNDECIDED with the planes to
//     redo in FP64.
__device__ __forceinline__ int post_cell(const DevParams &P, int np, float a0, float a1, float a2, float band,
                                         float &v, float &t1, float &t2) {
  v = t1 = t2 = 0.f;
  const int model = P.which_mc_model;
  if (model == 5) {
    v = a0;
    if (np > 2) { t1 = a1; t2 = a2; }
  } else if (model == 7) {
    v = sqrtf(a0 * a1);
  } else {
    // a nonzero thickness is at least one source's value at the cut; below
    // half of that only rounding residues of the tensor-core corner
    // subtraction remain: the reference's sum there is exactly 0
    t1 = a0 < P.kln_tzero ? 0.f : a0;
    t2 = a1 < P.kln_tzero ? 0.f : a1;
    // T/dT as T (1/dT): within 2 ulp of the quotient, inside the band
    const float di = t1 * P.kln_inv_dT_f, dj = t2 * P.kln_inv_dT_f;
    const float fi = di - floorf(di), fj = dj - floorf(dj);
    const float bi = fmaf(band, di, 1e-7f), bj = fmaf(band, dj, 1e-7f);
    const int tm = P.kln_tmax;
    const bool both = t1 > 0.f && t2 > 0.f;
    const bool near_a = t1 > 0.f && (fi < bi || fi > 1.f - bi) && (both || di > tm - 3);
    const bool near_b = t2 > 0.f && (fj < bj || fj > 1.f - bj) && (both || dj > tm - 3);
    if (near_a || near_b) return CELL_UNDECIDED | (near_a ? CELL_NEED_A : 0) | (near_b ? CELL_NEED_B : 0);
    if (di >= tm - 2 || dj >= tm - 2) return CELL_TABLE;
    // a zero thickness reads the zero first row / column of the table
    // (src/MCnucl.cpp:937-944): the interpolation is exactly 0 there
    if (!both) return CELL_OK;
    v = kln_interp(P, (int)di, (int)dj, fi, fj);
  }
  return CELL_OK;
}

// The thickness of plane `pl` (0: T_A, 1: T_B) at the cell (i, j) in FP64,
// summed as the reference sums it (MCnucl::setThickness,
// src/MCnucl.cpp:432-478; Particle::getSmoothTn, src/Particle.cpp:122-132):
// every thickness record of the plane whose window holds the cell adds
// peak exp(-r^2/2w^2) unless r > 5w (disk nucleons: 10/sigma_in unless
// dc > dsq, added one by one in FP64 as the reference adds them).  The
// plane's records are S[base, base + n), x-sorted, so those of row i sit in
// a few 32-record chunks.  Called by a whole warp (lanes over the records);
// every lane returns the sum.
__device__ __forceinline__ double thickness_fp64(const DevParams &P, const Source *S, int base, int n, int pl, int i,
                                                 int j) {
  const int lane = threadIdx.x & 31;
  // the chunks holding a record whose row window reaches row i: all window
  // rows loaded at once (independent loads), one bit per chunk
  constexpr int kMaxChunks = (kMaxA + 31) / 32;
  uint32_t chunks = 0;
#pragma unroll
  for (int c = 0; c < kMaxChunks; c++) {
    const int k = 32 * c + lane;
    const bool in = k < n && i >= S[base + k].xl && i < S[base + k].xr;
    if (__ballot_sync(0xffffffffu, in)) chunks |= 1u << c;
  }
  const double xg = __dadd_rn(P.xmin, __dmul_rn((double)i, P.dx));
  const double yg = __dadd_rn(P.ymin, __dmul_rn((double)j, P.dy));
  const double cut = __dmul_rn(5., P.width), cut2 = cut * cut;
  const double inv2w2 = 1.0 / (2.0 * P.w2);
  double sum = 0.0;
  int ndisk = 0;
  while (chunks) {
    const int c = __ffs(chunks) - 1;
    chunks &= chunks - 1u;
    const int k = 32 * c + lane;
    double t = 0.0;
    bool disk_hit = false;
    if (k < n) {
      const Source &s = S[base + k];
      if ((s.kind & 15) == SRC_THICK && s.plane == pl && i >= s.xl && i < s.xr && j >= s.yl && j < s.yr) {
        const double dc = sq_dist_rn(s.x, s.y, xg, yg);
        if (s.kind & 16) {
          disk_hit = !(dc > P.dsq);
        } else {
          // r = sqrt(dc) > 5w decided on dc away from the cut
          const bool keep = dc < cut2 * (1 - 1e-12) ? true
                            : dc > cut2 * (1 + 1e-12) ? false
                                                      : !(__dsqrt_rn(dc) > cut);
          if (keep) t = P.peak * exp(-dc * inv2w2);
        }
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    sum += __shfl_sync(0xffffffffu, t, 0);
    ndisk += __popc(__ballot_sync(0xffffffffu, disk_hit));
  }
  if (ndisk) {   // disk nucleons: n equal terms, added in turn
    const double c = 10.0 / P.sigin;
    for (int k = 0; k < ndisk; k++) sum += c;
  }
  return sum;
}

// The MC-KLN cell from thickness values taken as decided in FP64 (the
// planes redone in FP64, the others already decided by their FP32 value),
// the table cell as the reference takes it (di = T_A/dT in FP64,
// src/MCnucl.cpp:659-676); t1, t2 receive the thickness outputs.
__device__ __forceinline__ int kln_cell_fp64(const DevParams &P, double ta, double tb, float &v, float &t1,
                                             float &t2) {
  const double di = ta / P.kln_dT, dj = tb / P.kln_dT;
  t1 = (float)ta;
  t2 = (float)tb;
  v = 0.f;
  const int tm = P.kln_tmax;
  if (di >= tm - 2 || dj >= tm - 2) return CELL_TABLE;
  if (ta == 0.0 || tb == 0.0) return CELL_OK;
  const int ii = (int)floor(di), jj = (int)floor(dj);
  v = kln_interp(P, ii, jj, (float)(di - ii), (float)(dj - jj));
  return CELL_OK;
}

// a thread's centre-of-mass sums and the density sum before fluctuations
struct CmSums {
  KSum c0, c1, c2, pre;
};

// An MC-KLN cell that post_cell left undecided, held in a CTA's list until
// the end of its event: the cell, the planes to redo, the FP32 thickness
// values post_cell took, then the density before (v) and after (vout) the
// per-cell fluctuations
struct PendCell {
  int i, j, need;
  float t1, t2, v, vout;
};

// Appends an undecided cell to the event's list; false when the list is full
// (the caller then decides the cell on its own path).
__device__ __forceinline__ bool kln_defer(PendCell *list, int *count, int cap, int i, int j, int code, float t1,
                                          float t2) {
  const int slot = atomicAdd(count, 1);
  if (slot >= cap) return false;
  list[slot] = PendCell{i, j, (code >> 4) & 3, t1, t2, 0.f, 0.f};
  return true;
}

// The event's listed cells, decided from FP64 thickness sums of their
// flagged planes: the warps take the cells in turn (each a warp-wide FP64
// sum), lane 0 writes the cell's outputs and its values into the list.
template <int NWARPS>
static __device__ __noinline__ void kln_finish_listed(const DevParams &P, const EventRec &rec, const Source *S,
                                                  PendCell *list, int n, float *rho, float *ta, float *tb,
                                                  int *s_status) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, ny = P.ny;
  const int base0 = rec.nsplat - rec.npart1 - rec.npart2, base1 = base0 + rec.npart1;
  for (int q = wid; q < n; q += NWARPS) {
    const PendCell c = list[q];
    const double da = (c.need & 1) ? thickness_fp64(P, S, base0, rec.npart1, 0, c.i, c.j) : (double)c.t1;
    const double db = (c.need & 2) ? thickness_fp64(P, S, base1, rec.npart2, 1, c.i, c.j) : (double)c.t2;
    if (lane == 0) {
      float v, t1, t2;
      if (kln_cell_fp64(P, da, db, v, t1, t2) == CELL_TABLE) *s_status = 4;
      const size_t g = (size_t)c.i * ny + c.j;
      const float vout = P.nbd ? nbd_cell(P, rec.ev, (uint32_t)g, v, t1, t2) : v;
      rho[g] = vout;
      if (ta) ta[g] = t1;
      if (tb) tb[g] = t2;
      list[q].v = v;
      list[q].vout = vout;
    }
  }
}

// Adds the listed cells to one thread's centre-of-mass sums in cell order
// (so that the sums do not depend on the order the cells were listed in);
// the sums go in and come back by value.
static __device__ __noinline__ CmSums kln_add_listed(const PendCell *list, int n, int ny, const float *xg,
                                                     const float *yg, CmSums cs) {
  long long last = -1;
  for (int k = 0; k < n; k++) {
    long long best = LLONG_MAX;
    int at = -1;
    for (int q = 0; q < n; q++) {
      const long long key = (long long)list[q].i * ny + list[q].j;
      if (key > last && key < best) { best = key; at = q; }
    }
    last = best;
    const PendCell &c = list[at];
    cs.pre.add(c.v);
    if (c.vout != 0.f) {
      cs.c0.add(c.vout);
      cs.c1.add(xg[c.i] * c.vout);
      cs.c2.add(yg[c.j] * c.vout);
    }
  }
  return cs;
}

// Warp-wide completion of post_cell: every lane passes its cell (i, j),
// code and thickness values; the undecided cells of the warp are redone one
// at a time by the whole warp, each flagged plane from FP64 sums over its
// thickness records (MC-KLN records: [projectile participants][target
// participants] at the end of the splat records).  All 32 lanes call it.
__device__ __forceinline__ void kln_resolve_warp(const DevParams &P, const EventRec &rec, const Source *S, int i,
                                                 int j, int &code, float &v, float &t1, float &t2) {
  unsigned m = __ballot_sync(0xffffffffu, (code & CELL_UNDECIDED) != 0);
  const int lane = threadIdx.x & 31;
  const int base0 = rec.nsplat - rec.npart1 - rec.npart2, base1 = base0 + rec.npart1;
  while (m) {
    const int src = __ffs(m) - 1;
    m &= m - 1u;
    const int ci = __shfl_sync(0xffffffffu, i, src), cj = __shfl_sync(0xffffffffu, j, src);
    const int need = __shfl_sync(0xffffffffu, code, src);
    double ta = (double)__shfl_sync(0xffffffffu, t1, src), tb = (double)__shfl_sync(0xffffffffu, t2, src);
    if (need & CELL_NEED_A) ta = thickness_fp64(P, S, base0, rec.npart1, 0, ci, cj);
    if (need & CELL_NEED_B) tb = thickness_fp64(P, S, base1, rec.npart2, 1, ci, cj);
    if (lane == src) code = kln_cell_fp64(P, ta, tb, v, t1, t2);
  }
}

// Column interval [ja, jb) of row i that the reference includes for source
// g.  dc(j) is convex in j, so the included cells form one interval around
// the column nearest the source.
static __device__ __forceinline__ void row_interval(const DevParams &P, const GroupSrc &g, int i, float dx2, float lo,
                                             float hi, const float *yg, float inv_dy, float ymin_f, int &ja,
                                             int &jb) {
  const int wl = g.yl, wr = g.yr;
  auto dcf = [&](int j) {
    float dy = yg[j] - g.yf;
    return fmaf(dy, dy, dx2);
  };
  auto inside = [&](int j) {
    float d = dcf(j);
    if (d < lo) return true;
    if (d > hi) return false;
    return cell_in_exact(P, g.x, g.y, g.kind, i, j);
  };
  ja = jb = wl;
  if (wr <= wl) return;
  float h2 = lo - dx2;
  int a, b;
  if (h2 > 0.f) {
    float h = sqrtf(h2);
    a = (int)ceilf((g.yf - h - ymin_f) * inv_dy);
    b = (int)floorf((g.yf + h - ymin_f) * inv_dy) + 1;
    a = max(a, wl);
    b = min(b, wr);
    // shrink to cells certainly inside (rounding of the estimate)
    while (a < b && !(dcf(a) < lo)) a++;
    while (b > a && !(dcf(b - 1) < lo)) b--;
  } else {
    a = b = 0;
  }
  if (a >= b) {
    // no certainly-inside cell: only the cells nearest the source can be in
    int jc = (int)floorf((g.yf - ymin_f) * inv_dy);
    a = b = -1;
    for (int j = max(wl, jc - 1); j <= min(wr - 1, jc + 2); j++) {
      if (inside(j)) {
        if (a < 0) a = j;
        b = j + 1;
      }
    }
    if (a < 0) return;
  }
  // extend by cells decided inside at the FP32 error scale
  while (a - 1 >= wl && inside(a - 1)) a--;
  while (b < wr && inside(b)) b++;
  ja = a;
  jb = b;
}

// Column interval [ja, jb) of row i inside the cut of a Gaussian source at
// (sxf, syf) (FP32 copy of the FP64 position *sxy) within the window
// columns [wl, wr): the same decision as row_interval, with scalar
// arguments so that it inlines.  dc(j) is convex in j, so the included
// cells form one interval around the column nearest the source; the FP32
// distance decides every cell except those within its error of the cut,
// which take the reference's FP64 test.
__device__ __forceinline__ void cut_interval(const DevParams &P, const double *sxy, int kind, float syf, int i,
                                             float dx2, float lo, float hi, const float *yg, float inv_dy,
                                             float ymin_f, int wl, int wr, int &ja, int &jb) {
  auto dcf = [&](int j) {
    const float dy = yg[j] - syf;
    return fmaf(dy, dy, dx2);
  };
  auto inside = [&](int j) {
    const float d = dcf(j);
    if (d < lo) return true;
    if (d > hi) return false;
    return cell_in_exact(P, sxy[0], sxy[1], kind, i, j);
  };
  ja = jb = wl;
  if (wr <= wl) return;
  int a, b;
  const float h2 = lo - dx2;
  if (h2 > 0.f) {
    const float h = sqrtf(h2);
    a = max((int)ceilf((syf - h - ymin_f) * inv_dy), wl);
    b = min((int)floorf((syf + h - ymin_f) * inv_dy) + 1, wr);
    while (a < b && !(dcf(a) < lo)) a++;
    while (b > a && !(dcf(b - 1) < lo)) b--;
  } else {
    a = b = 0;
  }
  if (a >= b) {
    const int jc = (int)floorf((syf - ymin_f) * inv_dy);
    a = b = -1;
    for (int j = max(wl, jc - 1); j <= min(wr - 1, jc + 2); j++) {
      if (inside(j)) {
        if (a < 0) a = j;
        b = j + 1;
      }
    }
    if (a < 0) return;
  }
  while (a - 1 >= wl && inside(a - 1)) a--;
  while (b < wr && inside(b)) b++;
  ja = a;
  jb = b;
}

// The hot-spot region of dumpEccentricities as a bit mask over the grid
// (one bit per cell, rows of ceil(ny/32) words): the union of the
// participant boxes on the reference's lattice (ranges mx0..my1 of the
// participant sources, src/MakeDensity.cpp:2341-2359).  NT: threads of the
// block (0: blockDim.x).
template <int NT>
__device__ __forceinline__ void hotspot_mask(const DevParams &P, const EventRec &rec, const Source *S, uint32_t *mask) {
  const int tid = threadIdx.x;
  const int nt = NT > 0 ? NT : (int)blockDim.x;
  const int nx = P.nx, ny = P.ny;
  const int nw = (ny + 31) / 32;
  for (int k = tid; k < nx * nw; k += nt) mask[k] = 0;
  __syncthreads();
  // sources in chunks of 32 per warp; the lanes then take the (source, row)
  // pairs of the chunk's boxes, so that all lanes set bits
  const int lane = tid & 31;
  for (int s0 = (tid >> 5) * 32; s0 < rec.nsrc; s0 += nt) {
    int r0 = 0, r1 = 0, c0 = 0, c1 = 0;
    if (s0 + lane < rec.nsrc) {
      const Source &src = S[s0 + lane];
      const int kd = src.kind & 15;
      if (kd == SRC_PART_BOX || kd == 3) {
        r0 = max(0, (int)src.mx0); r1 = min(nx, (int)src.mx1);
        c0 = max(0, (int)src.my0); c1 = min(ny, (int)src.my1);
        if (r1 <= r0 || c1 <= c0) r1 = r0;
      } else {
        r1 = r0;
      }
    }
    // exclusive prefix of the row counts over the chunk
    const int nr = r1 - r0;
    int pre = nr;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, pre, o);
      if (lane >= o) pre += t;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 31);
    pre -= nr;
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      // the box of pair t: the last lane whose prefix is <= t
      int src_lane = 0;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const int cand = src_lane + o;
        const int pc = __shfl_sync(0xffffffffu, pre, cand);
        if (pc <= t) src_lane = cand;
      }
      const int br0 = __shfl_sync(0xffffffffu, r0, src_lane), bpre = __shfl_sync(0xffffffffu, pre, src_lane);
      const int bc0 = __shfl_sync(0xffffffffu, c0, src_lane), bc1 = __shfl_sync(0xffffffffu, c1, src_lane);
      if (t < total) {
        const int row = br0 + (t - bpre);
        for (int wd = bc0 >> 5; wd <= (bc1 - 1) >> 5; wd++) {
          const int lo = max(bc0, wd * 32), hi = min(bc1, wd * 32 + 32);
          const uint32_t bits = (hi - lo >= 32) ? 0xffffffffu : (((1u << (hi - lo)) - 1u) << (lo - wd * 32));
          atomicOr(&mask[row * nw + wd], bits);
        }
      }
    }
  }
  __syncthreads();
}

// The eccentricity pass of dumpEccentricities over the event's density
// (centre of mass already known: xo, yo are the grid coordinates relative
// to it).  NT: threads of the block (0: blockDim.x).
template <int LO, int HI, int NT>
__device__ __noinline__ void moments(const DevParams &P, const EventRec &rec, const Source *S, const float *rho, uint32_t *mask,
                        const float *xo, const float *yo, float2 *red, double tot0, double *ecc_out) {
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int nt = NT > 0 ? NT : (int)blockDim.x, nwarps = nt / 32;
  const int ny = P.ny;
  const int nw = (ny + 31) / 32;
  // ---- eccentricity mask from the participant boxes
  hotspot_mask<NT>(P, rec, S, mask);

  constexpr int NO = HI - LO + 1;
  float a_rn[10];
  float a_norm = 0.f;
  float a_re2[NO], a_im2[NO], a_ren[NO], a_imn[NO], a_np[NO];
#pragma unroll
  for (int k = 0; k < 10; k++) a_rn[k] = 0.f;
#pragma unroll
  for (int k = 0; k < NO; k++) a_re2[k] = a_im2[k] = a_ren[k] = a_imn[k] = a_np[k] = 0.f;
  const int from = P.ecc_from, to = P.ecc_to;
  // warps take (row, 32-column block) items of the bounding box, lanes the
  // columns; blocks aligned to 32 columns (one mask word per item)
  const int jlo = rec.jmin & ~31;
  const int nbj = rec.jmax > rec.jmin ? (rec.jmax - jlo + 31) >> 5 : 0;
  const int nitem = rec.imax > rec.imin ? (rec.imax - rec.imin) * nbj : 0;
  // the next item's density is loaded before the current one is processed;
  // (ib, jb): row and column block of the warp's next item
  int ib = nbj > 0 ? wid / nbj : 0, jb = wid - ib * nbj;
  auto fetch = [&](int c, int &i, int &j) -> float {
    float v = 0.f;
    if (c < nitem) {
      i = rec.imin + ib;
      j = jlo + (jb << 5) + lane;
      if (j >= rec.jmin && j < rec.jmax) v = rho[(size_t)i * ny + j];
    }
    jb += nwarps;   // nbj >= 1 whenever there are items: at most nwarps steps
    if (nbj > 0)
      while (jb >= nbj) { jb -= nbj; ib++; }
    return v;
  };
  int i_next = 0, j_next = 0;
  float d_next = fetch(wid, i_next, j_next);
  for (int c = wid; c < nitem; c += nwarps) {
    const int i = i_next, j = j_next;
    const float d = d_next;
    d_next = fetch(c + nwarps, i_next, j_next);
    if (d == 0.f) continue;
    float x = xo[i], y = yo[j];
    float r2 = x * x + y * y;
    float r = sqrtf(r2);
    float rp[10];
    rp[0] = 1.f;
#pragma unroll
    for (int k = 1; k < 10; k++) rp[k] = rp[k - 1] * r;
#pragma unroll
    for (int k = 1; k < 10; k++) a_rn[k] += rp[k] * d;
    bool imp = (mask[i * nw + (j >> 5)] >> (j & 31)) & 1u;
    if (!imp) continue;
    // 1/r only enters the r^2-weighted sums of orders >= 3 (approximate
    // reciprocal square root, 2^-22 relative)
    const float inv_r = r2 > 0.f ? rsqrtf(r2) : 0.f;
    a_norm += r2 * d;
    float zr = x, zi = y;   // z^n
#pragma unroll
    for (int n = 1; n <= HI; n++) {
      if (n > 1) {
        float t = zr * x - zi * y;
        zi = zr * y + zi * x;
        zr = t;
      }
      if (n >= LO && n >= from && n <= to) {
        const int q = n - LO;
        // r^2 e^{in theta} = z^n r^{2-n};  r^n e^{in theta} = z^n (r^3 e^{i theta} for n = 1).
        // n = 2: the r^2 and r^n sums coincide (taken from a_ren, a_imn and a_norm below)
        if (n == 1) {
          a_re2[q] += zr * r * d;
          a_im2[q] += zi * r * d;
          a_ren[q] += zr * r2 * d;
          a_imn[q] += zi * r2 * d;
          a_np[q] += rp[3] * d;
        } else {
          if (n > 2) {
            float s2 = inv_r;
#pragma unroll
            for (int k = 3; k < n; k++) s2 *= inv_r;
            const float sd = s2 * d;
            a_re2[q] += zr * sd;
            a_im2[q] += zi * sd;
            a_np[q] += rp[n] * d;
          }
          a_ren[q] += zr * d;
          a_imn[q] += zi * d;
        }
      }
    }
  }
  if (LO <= 2 && HI >= 2) {   // order 2: r^2 e^{2i theta} = z^2, and r^2 = r2
    a_re2[2 - LO] = a_ren[2 - LO];
    a_im2[2 - LO] = a_imn[2 - LO];
    a_np[2 - LO] = a_norm;
  }
  // ---- block reduction in double-float (each accumulator retires as it is reduced)
  constexpr int NV = 10 + 5 * NO;
  auto put = [&](int k, float x) {
    DF t = df_warp_sum(DF{x, 0.f});
    if (lane == 0) red[wid * 64 + k] = make_float2(t.hi, t.lo);
  };
#pragma unroll
  for (int k = 1; k < 10; k++) put(k - 1, a_rn[k]);
  put(9, a_norm);
#pragma unroll
  for (int q = 0; q < NO; q++) {
    put(10 + 5 * q, a_re2[q]);
    put(11 + 5 * q, a_im2[q]);
    put(12 + 5 * q, a_ren[q]);
    put(13 + 5 * q, a_imn[q]);
    put(14 + 5 * q, a_np[q]);
  }
  __syncthreads();
  __shared__ double s_tot[64];
  if (tid < NV) {
    double t = 0;
    for (int w = 0; w < nwarps; w++) t += (double)red[w * 64 + tid].x + (double)red[w * 64 + tid].y;
    s_tot[tid] = t;
  }
  __syncthreads();
  // output k of the event's row (one division per thread):
  // 5 (n - 1) + c, c < 4: the eps_n components, c = 4: <r^n>; 45..48 the totals
  if (tid < kEccLen) {
    const double *tot = s_tot;
    const double ff = P.final_factor, eps = 1e-15;
    const double dn = tot0;
    // an all-zero density (possible after NBD fluctuations) has no centre of
    // mass: the reference's sums are then NaN (0 * NaN), as here
    const bool empty = !(dn > 0);
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    double v = 0.0;
    if (tid < 45) {
      const int n = tid / 5 + 1, c = tid - 5 * (n - 1);
      if (c == 4) {
        v = empty ? nan : (tot[n - 1] * ff) / (dn * ff);
      } else if (n >= LO && n <= HI && n >= from && n <= to) {
        const int q = n - LO;
        const double den = c < 2 ? tot[9] * ff + eps : tot[14 + 5 * q] * ff + eps;
        v = empty ? nan : -(tot[10 + 5 * q + c] * ff) / den;
      }
    } else if (tid == 45) {
      v = (double)(rec.npart1 + rec.npart2);
    } else if (tid == 46) {
      v = (double)rec.ncoll;
    } else if (tid == 47) {
      v = tot0 * ff * P.dx * P.dy;
    } else {
      v = rec.b;
    }
    ecc_out[tid] = v;
  }
  __syncthreads();
}


}  // namespace smc
