// Stage 2 of the event pipeline: thickness / density splat and the
// eccentricity moments, one CTA per event.
//
// Reference behaviour restated here:
//   T_A, T_B (Gaussian nucleons, r <= 5w)     src/MCnucl.cpp:432-478, src/Particle.cpp:122-132
//   Glauber rho = (1-a)/2 WN + a BC            src/MCnucl.cpp:688-779, :822-866
//   sqrt(T_A T_B) scaling                      src/MCnucl.cpp:780-811
//   MC-KLN per-cell table lookup               src/MCnucl.cpp:654-687, src/arsenal.cpp:33-54
//   centre of mass, <r^n>, eps_n over the hot-spot mask
//                                              src/MakeDensity.cpp:2244-2511
//
// The grid is processed in strips of kR rows held in shared memory.  For a
// group of sources reaching the strip, one thread per (source, row) pair
// computes the row factor w exp(-dx^2/2w^2) and the exact column interval of
// the cells the reference includes (window and r <= 5w / dc <= 25w^2 /
// dc <= dsq cut): FP32 away from the cut, FP64 rounded as the reference
// rounds for the one cell per side that can sit within the FP32 error of
// it.  Column factors exp(-dy^2/2w^2) are computed once per (source,
// column).  Each warp then owns kRW rows of the strip and adds its
// sources' rows with plain shared-memory read-modify-writes (no atomics).
// All reductions run in FP32 pairs (double-float): FP64 arithmetic is rare
// on this part and used only for the per-event totals.
#include "smc_device.cuh"
#include "smc_kernels.h"

namespace smc {

constexpr int kGT = 512;            // threads per CTA
constexpr int kWarps = kGT / 32;
constexpr int kRW = 2;              // rows per warp
constexpr int kR = kWarps * kRW;    // rows per strip
constexpr int kGS = 64;             // sources per group

struct GroupSrc {
  double x, y;
  float xf, yf, weight;
  int16_t xl, xr, yl, yr;
  int16_t kind, plane;
};

struct PairDat {      // one (source, row) pair of a strip
  float exw;          // weight * exp(-dx^2 / 2w^2)
  int16_t ja, jb;     // included columns [ja, jb)
};

struct GridLayout {
  int nyp, mw, np;
  size_t off_acc, off_list, off_grp, off_pair, off_ey, off_xg, off_yg, off_red, total;
};

__host__ __device__ inline GridLayout grid_layout(int nx, int ny, int mw, int np) {
  GridLayout L;
  L.nyp = (ny + 31) / 32 * 32;
  L.mw = mw;
  L.np = np;
  size_t o = 0;
  L.off_acc = o; o += sizeof(float) * np * kR * L.nyp;
  size_t mask_bytes = sizeof(uint32_t) * (size_t)nx * (L.nyp / 32);
  if (mask_bytes > o) o = mask_bytes;   // the eccentricity mask reuses the accumulators
  o = (o + 15) / 16 * 16;
  L.off_list = o; o += sizeof(int) * kGT;
  o = (o + 15) / 16 * 16;
  L.off_grp = o; o += sizeof(GroupSrc) * kGS;
  L.off_pair = o; o += sizeof(PairDat) * kGS * kR;
  L.off_ey = o; o += sizeof(float) * kGS * mw;
  o = (o + 15) / 16 * 16;
  L.off_xg = o; o += sizeof(float) * 2 * nx;   // grid x, then x - x_cm
  L.off_yg = o; o += sizeof(float) * 2 * L.nyp;
  o = (o + 15) / 16 * 16;
  L.off_red = o; o += sizeof(float2) * kWarps * 64;
  L.total = o;
  return L;
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

// exact per-cell inclusion, FP64 as the reference evaluates it
__device__ __noinline__ bool cell_in_exact(const DevParams &P, double sx, double sy, int kind, int i, int j) {
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

// Column interval [ja, jb) of row i that the reference includes for source
// g.  dc(j) is convex in j, so the included cells form one interval around
// the column nearest the source.
__device__ __noinline__ void row_interval(const DevParams &P, const GroupSrc &g, int i, float dx2, float lo,
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

template <int LO, int HI>
__device__ __noinline__ void moments(const DevParams &P, const EventRec &rec, const Source *S, const float *rho, uint32_t *mask,
                        const float *xo, const float *yo, float2 *red, double tot0, double *ecc_out) {
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int nx = P.nx, ny = P.ny;
  const int nw = (ny + 31) / 32;
  // ---- eccentricity mask from the participant boxes
  for (int k = tid; k < nx * nw; k += kGT) mask[k] = 0;
  __syncthreads();
  for (int s = tid; s < rec.nsrc; s += kGT) {
    const Source &src = S[s];
    int kd = src.kind & 15;
    if (kd != SRC_PART_BOX && kd != 3) continue;
    int r0 = max(0, (int)src.mx0), r1 = min(nx, (int)src.mx1);
    int c0 = max(0, (int)src.my0), c1 = min(ny, (int)src.my1);
    if (r1 <= r0 || c1 <= c0) continue;
    int w0 = c0 >> 5, w1 = (c1 - 1) >> 5;
    for (int row = r0; row < r1; row++)
      for (int wd = w0; wd <= w1; wd++) {
        int lo = max(c0, wd * 32), hi = min(c1, wd * 32 + 32);
        uint32_t bits = (hi - lo >= 32) ? 0xffffffffu : (((1u << (hi - lo)) - 1u) << (lo - wd * 32));
        atomicOr(&mask[row * nw + wd], bits);
      }
  }
  __syncthreads();

  constexpr int NO = HI - LO + 1;
  float a_rn[10];
  float a_norm = 0.f;
  float a_re2[NO], a_im2[NO], a_ren[NO], a_imn[NO], a_np[NO];
#pragma unroll
  for (int k = 0; k < 10; k++) a_rn[k] = 0.f;
#pragma unroll
  for (int k = 0; k < NO; k++) a_re2[k] = a_im2[k] = a_ren[k] = a_imn[k] = a_np[k] = 0.f;
  const int from = P.ecc_from, to = P.ecc_to;
  const int bi = rec.imax - rec.imin, bj = rec.jmax - rec.jmin;
  const int ncell = bi > 0 && bj > 0 ? bi * bj : 0;
  for (int c = tid; c < ncell; c += kGT) {
    int i = rec.imin + c / bj, j = rec.jmin + c % bj;
    float d = rho[(size_t)i * ny + j];
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
    float inv_r = r > 0.f ? 1.f / r : 0.f;
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
        // r^2 e^{in theta} = z^n r^{2-n};  r^n e^{in theta} = z^n (r^3 e^{i theta} for n = 1)
        float s2 = n == 1 ? r : 1.f;
#pragma unroll
        for (int k = 2; k < n; k++) s2 *= inv_r;
        a_re2[q] += zr * s2 * d;
        a_im2[q] += zi * s2 * d;
        if (n == 1) {
          a_ren[q] += zr * r2 * d;
          a_imn[q] += zi * r2 * d;
          a_np[q] += rp[3] * d;
        } else {
          a_ren[q] += zr * d;
          a_imn[q] += zi * d;
          a_np[q] += rp[n] * d;
        }
      }
    }
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
    for (int w = 0; w < kWarps; w++) t += (double)red[w * 64 + tid].x + (double)red[w * 64 + tid].y;
    s_tot[tid] = t;
  }
  __syncthreads();
  if (tid == 0) {
    const double *tot = s_tot;
    const double ff = P.final_factor, eps = 1e-15;
    double *out = ecc_out;
    const double dn = tot0;
    for (int n = 1; n < 10; n++) {
      double *o = out + 5 * (n - 1);
      o[0] = o[1] = o[2] = o[3] = 0.0;
      o[4] = (tot[n - 1] * ff) / (dn * ff);
      if (n >= LO && n <= HI && n >= from && n <= to) {
        int q = n - LO;
        o[0] = -(tot[10 + 5 * q] * ff) / (tot[9] * ff + eps);
        o[1] = -(tot[11 + 5 * q] * ff) / (tot[9] * ff + eps);
        o[2] = -(tot[12 + 5 * q] * ff) / (tot[14 + 5 * q] * ff + eps);
        o[3] = -(tot[13 + 5 * q] * ff) / (tot[14 + 5 * q] * ff + eps);
      }
    }
    out[45] = (double)(rec.npart1 + rec.npart2);
    out[46] = (double)rec.ncoll;
    out[47] = tot0 * ff * P.dx * P.dy;
    out[48] = rec.b;
  }
  __syncthreads();
}

template <int LO, int HI>
__global__ void __launch_bounds__(kGT) k_grid(DevParams P, int n_events, const EventRec *recs, const Source *srcs,
                                              float *out_rho, float *out_ta, float *out_tb, float *scratch,
                                              double *out_ecc, int *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridLayout L = grid_layout(P.nx, P.ny, P.splat_mw, P.n_planes);
  float *acc = reinterpret_cast<float *>(smem + L.off_acc);
  int *list = reinterpret_cast<int *>(smem + L.off_list);
  GroupSrc *grp = reinterpret_cast<GroupSrc *>(smem + L.off_grp);
  PairDat *pairs = reinterpret_cast<PairDat *>(smem + L.off_pair);
  float *eyb = reinterpret_cast<float *>(smem + L.off_ey);
  float *xg = reinterpret_cast<float *>(smem + L.off_xg);
  float *yg = reinterpret_cast<float *>(smem + L.off_yg);
  float2 *red = reinterpret_cast<float2 *>(smem + L.off_red);
  __shared__ int s_status;
  __shared__ double s_cm[3];

  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int nx = P.nx, ny = P.ny, nyp = L.nyp, mw = L.mw, np = L.np;
  const float inv2w2 = (float)(1.0 / (2.0 * P.w2));
  const float lim = (float)(25.0 * P.w2), lim_lo = lim * (1.f - 1e-4f), lim_hi = lim * (1.f + 1e-4f);
  const float dsq = (float)P.dsq, dsq_lo = dsq * (1.f - 1e-4f), dsq_hi = dsq * (1.f + 1e-4f);
  const float inv_dy = (float)(1.0 / P.dy), ymin_f = (float)P.ymin;
  const int model = P.which_mc_model;

  for (int i = tid; i < nx; i += kGT) xg[i] = (float)(P.xmin + i * P.dx);
  for (int j = tid; j < ny; j += kGT) yg[j] = (float)(P.ymin + j * P.dy);

  for (int e = blockIdx.x; e < n_events; e += gridDim.x) {
    const EventRec rec = recs[e];
    const Source *S = srcs + (size_t)e * P.max_src;
    float *rho = out_rho ? out_rho + (size_t)e * nx * ny : scratch + (size_t)blockIdx.x * nx * ny;
    float *ta = out_ta ? out_ta + (size_t)e * nx * ny : nullptr;
    float *tb = out_tb ? out_tb + (size_t)e * nx * ny : nullptr;
    if (tid == 0) s_status = rec.status;
    KSum cm0, cm1, cm2;
    __syncthreads();

    for (int r0 = 0; r0 < nx; r0 += kR) {
      const int rows = min(kR, nx - r0);
      const bool active = r0 + rows > rec.imin && r0 < rec.imax;
      if (active) {
        for (int k = tid; k < np * kR * nyp; k += kGT) acc[k] = 0.f;
        for (int c0 = 0; c0 < rec.nsrc; c0 += kGT) {
          // compact the sources of this chunk that reach the strip
          int k = c0 + tid;
          bool hit = false;
          if (k < rec.nsrc) {
            const Source &s = S[k];
            hit = s.xl < r0 + rows && s.xr > r0 && s.yr > s.yl && (s.kind & 15) != 3;
          }
          unsigned bal = __ballot_sync(0xffffffffu, hit);
          __syncthreads();
          if (lane == 0) list[kGT - 1 - wid] = __popc(bal);
          __syncthreads();
          int off = 0, tot = 0;
          for (int q = 0; q < kWarps; q++) {
            int cq = list[kGT - 1 - q];
            off += q < wid ? cq : 0;
            tot += cq;
          }
          __syncthreads();
          if (hit) list[off + __popc(bal & ((1u << lane) - 1u))] = k;
          __syncthreads();
          for (int g0 = 0; g0 < tot; g0 += kGS) {
            const int gn = min(kGS, tot - g0);
            for (int t = tid; t < gn; t += kGT) {
              const Source &s = S[list[g0 + t]];
              GroupSrc g;
              g.x = s.x; g.y = s.y; g.xf = (float)s.x; g.yf = (float)s.y; g.weight = s.weight;
              // the column table holds mw columns per source: a window never reaches past it
              g.xl = s.xl; g.xr = s.xr; g.yl = s.yl; g.yr = (int16_t)min((int)s.yr, (int)s.yl + mw);
              g.kind = s.kind; g.plane = s.plane;
              grp[t] = g;
            }
            __syncthreads();
            // column factors, one per (source, column)
            for (int t = tid; t < gn * mw; t += kGT) {
              int q = t / mw, c = t - q * mw;
              const GroupSrc &g = grp[q];
              int j = g.yl + c;
              float v = 0.f;
              if (j < g.yr) {
                float dy = yg[j] - g.yf;
                v = (g.kind & 16) ? 1.f : __expf(-dy * dy * inv2w2);
              }
              eyb[t] = v;
            }
            // row factors and included column intervals, one per (source, row)
            for (int t = tid; t < gn * kR; t += kGT) {
              int q = t / kR, r = t - q * kR;
              const GroupSrc &g = grp[q];
              const int i = r0 + r;
              PairDat pd;
              pd.exw = 0.f;
              pd.ja = pd.jb = 0;
              if (r < rows && i >= g.xl && i < g.xr) {
                const bool disk = g.kind & 16;
                const float dx = xg[i] - g.xf, dx2 = dx * dx;
                pd.exw = disk ? g.weight : g.weight * __expf(-dx2 * inv2w2);
                int ja, jb;
                row_interval(P, g, i, dx2, disk ? dsq_lo : lim_lo, disk ? dsq_hi : lim_hi, yg, inv_dy, ymin_f, ja,
                             jb);
                pd.ja = (int16_t)ja;
                pd.jb = (int16_t)jb;
              }
              pairs[t] = pd;
            }
            __syncthreads();
            // accumulation: warp wid owns rows wid*kRW .. wid*kRW+kRW-1 of the strip
#pragma unroll
            for (int rr = 0; rr < kRW; rr++) {
              const int r = wid * kRW + rr;
              if (r >= rows) continue;
              for (int q = 0; q < gn; q++) {
                const PairDat pd = pairs[q * kR + r];
                if (pd.ja >= pd.jb) continue;
                const int yl = grp[q].yl, pl = grp[q].plane;
                float *arow = acc + ((size_t)pl * kR + r) * nyp;
                const float *ey = eyb + q * mw - yl;
                for (int j = pd.ja + lane; j < pd.jb; j += 32) arow[j] += pd.exw * ey[j];
              }
            }
            __syncthreads();
          }
        }
      }
      // post-op per cell, outputs and centre-of-mass sums
      for (int c = tid; c < rows * ny; c += kGT) {
        const int rr = c / ny, j = c - rr * ny, i = r0 + rr;
        float v = 0.f, t1 = 0.f, t2 = 0.f;
        if (active) {
          const float a0 = acc[rr * nyp + j];
          const float a1 = np > 1 ? acc[(kR + rr) * nyp + j] : 0.f;
          if (model == 5) {
            v = a0;
            if (np > 2) { t1 = a1; t2 = acc[(2 * kR + rr) * nyp + j]; }
          } else if (model == 7) {
            v = sqrtf(a0 * a1);
          } else {   // MC-KLN: planes hold T_A, T_B
            t1 = a0; t2 = a1;
            float di = t1 / (float)P.kln_dT, dj = t2 / (float)P.kln_dT;
            const int tm = P.kln_tmax;
            if (di < 0.f || di >= tm - 2 || dj < 0.f || dj >= tm - 2) {
              s_status = 4;
            } else {
              int ii = (int)floorf(di), jj = (int)floorf(dj);
              const float *T = P.kln_table;
              v = six_point(di - ii, dj - jj, T[ii * tm + jj], T[ii * tm + jj + 1], T[ii * tm + jj + 2],
                            T[(ii + 1) * tm + jj], T[(ii + 1) * tm + jj + 1], T[(ii + 2) * tm + jj]);
            }
          }
        }
        rho[(size_t)i * ny + j] = v;
        if (ta) ta[(size_t)i * ny + j] = t1;
        if (tb) tb[(size_t)i * ny + j] = t2;
        if (v != 0.f) {
          cm0.add(v);
          cm1.add(xg[i] * v);
          cm2.add(yg[j] * v);
        }
      }
      __syncthreads();
    }
    // ---- centre of mass
    {
      DF a = df_warp_sum(cm0.df()), b = df_warp_sum(cm1.df()), c = df_warp_sum(cm2.df());
      if (lane == 0) {
        red[wid * 64] = make_float2(a.hi, a.lo);
        red[wid * 64 + 1] = make_float2(b.hi, b.lo);
        red[wid * 64 + 2] = make_float2(c.hi, c.lo);
      }
      __syncthreads();
      if (tid == 0) {
        double sa = 0, sb = 0, sc = 0;
        for (int w = 0; w < kWarps; w++) {
          sa += (double)red[w * 64].x + (double)red[w * 64].y;
          sb += (double)red[w * 64 + 1].x + (double)red[w * 64 + 1].y;
          sc += (double)red[w * 64 + 2].x + (double)red[w * 64 + 2].y;
        }
        s_cm[0] = sa; s_cm[1] = sb / sa; s_cm[2] = sc / sa;
        if (!(sa * P.dx * P.dy >= 1e-15) && s_status == 0) s_status = 5;   // MCnucl.cpp:812-816
      }
      __syncthreads();
    }
    const double xc = s_cm[1], yc = s_cm[2], tot0 = s_cm[0];
    float *xo = xg + nx;
    float *yo = yg + nyp;
    for (int i = tid; i < nx; i += kGT) xo[i] = (float)((P.xmin + i * P.dx) - xc);
    for (int j = tid; j < ny; j += kGT) yo[j] = (float)((P.ymin + j * P.dy) - yc);
    __syncthreads();
    if (!P.no_moments)
      moments<LO, HI>(P, rec, S, rho, reinterpret_cast<uint32_t *>(acc), xo, yo, red, tot0,
                      out_ecc + (size_t)e * kEccLen);
    if (tid == 0 && status) status[e] = s_status;
    __syncthreads();
  }
}

size_t grid_smem(const DevParams &P) { return grid_layout(P.nx, P.ny, P.splat_mw, P.n_planes).total; }

int grid_blocks_per_sm(const DevParams &P) {
  const bool narrow = P.ecc_from >= 2 && P.ecc_to <= 5;
  const void *k = narrow ? (const void *)k_grid<2, 5> : (const void *)k_grid<1, 9>;
  size_t smem = grid_smem(P);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
  int nb = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kGT, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

cudaError_t launch_grid(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs, float *out_rho,
                        float *out_ta, float *out_tb, float *scratch, double *out_ecc, int *status, int grid,
                        cudaStream_t st) {
  size_t smem = grid_smem(P);
  const bool narrow = P.ecc_from >= 2 && P.ecc_to <= 5;
  auto kern = narrow ? k_grid<2, 5> : k_grid<1, 9>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kGT, smem, st>>>(P, n_events, recs, srcs, out_rho, out_ta, out_tb, scratch, out_ecc, status);
  return cudaGetLastError();
}

}  // namespace smc
