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
// The grid is processed in strips of kR rows.  Each warp owns one row of the
// strip, so accumulation into shared memory needs no atomics; the column
// factors exp(-(y_j-y_s)^2/2w^2) of a group of sources are computed once per
// strip.  Window edges were computed exactly in stage 1; the per-cell cut
// (r <= 5w, dc <= 25 w^2, dc <= dsq) is decided in FP32 away from the
// threshold and in FP64, rounded as the reference rounds, near it.
#include "smc_device.cuh"
#include "smc_kernels.h"

namespace smc {

constexpr int kGT = 512;   // threads per CTA
constexpr int kR = kGT / 32;  // rows per strip (one per warp)
constexpr int kGS = 128;   // sources per column-factor group

struct GroupSrc {
  double x, y;
  float xf, yf, weight;
  int16_t xl, xr, yl, yr;
  int16_t kind, plane;
};

struct GridLayout {
  int nyp;      // padded row length
  int mw;       // max window width in columns
  size_t off_acc, off_list, off_grp, off_ey, off_xg, off_yg, off_red, total;
};

__host__ __device__ inline GridLayout grid_layout(int nx, int ny, int mw) {
  GridLayout L;
  L.nyp = (ny + 31) / 32 * 32;
  L.mw = mw;
  size_t o = 0;
  L.off_acc = o; o += sizeof(float) * 3 * kR * L.nyp;
  size_t mask_bytes = sizeof(uint32_t) * (size_t)nx * (L.nyp / 32);
  if (mask_bytes > o) o = mask_bytes;   // the eccentricity mask reuses the accumulators
  o = (o + 15) / 16 * 16;
  L.off_list = o; o += sizeof(int) * kGT;
  o = (o + 15) / 16 * 16;
  L.off_grp = o; o += sizeof(GroupSrc) * kGS;
  L.off_ey = o; o += sizeof(float) * kGS * mw;
  o = (o + 15) / 16 * 16;
  L.off_xg = o; o += sizeof(float) * 2 * nx;   // grid x, then x - x_cm
  L.off_yg = o; o += sizeof(float) * 2 * L.nyp;
  o = (o + 15) / 16 * 16;
  L.off_red = o; o += sizeof(double) * (kGT / 32) * 64;
  L.total = o;
  return L;
}

// exact per-cell inclusion, FP64 as the reference evaluates it
__device__ __noinline__ bool cell_in_exact(const DevParams &P, const GroupSrc &g, int i, int j) {
  double xg = __dadd_rn(P.xmin, __dmul_rn((double)i, P.dx));
  double yg = __dadd_rn(P.ymin, __dmul_rn((double)j, P.dy));
  double dc = sq_dist_rn(g.x, g.y, xg, yg);
  int k = g.kind & 15;
  if (g.kind & 16) return !(dc > P.dsq);                      // disk nucleons / entropy
  if (k == SRC_COLL) return dc <= __dmul_rn(25., P.w2);       // MCnucl.cpp:754
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

template <int LO, int HI>
__device__ void moments(const DevParams &P, const EventRec &rec, const Source *S, const float *rho, uint32_t *mask,
                        const float *xo, const float *yo, double *red, double xc_sum[3], double *ecc_out) {
  const int tid = threadIdx.x;
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
    for (int k = 0; k < 10; k++) a_rn[k] += rp[k] * d;
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
      if (n >= LO) {
        const int q = n - LO;
        if (n >= from && n <= to) {
          // r^2 e^{in theta} = z^n r^{2-n};  r^n e^{in theta} = z^n (r^3 e^{i theta} for n = 1)
          float s2 = 1.f;
          if (n == 1) s2 = r;
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
  }
  // ---- block reduction in FP64
  constexpr int NV = 11 + 5 * NO;
  double v[NV];
#pragma unroll
  for (int k = 0; k < 10; k++) v[k] = a_rn[k];
  v[10] = a_norm;
#pragma unroll
  for (int q = 0; q < NO; q++) {
    v[11 + 5 * q] = a_re2[q]; v[12 + 5 * q] = a_im2[q]; v[13 + 5 * q] = a_ren[q];
    v[14 + 5 * q] = a_imn[q]; v[15 + 5 * q] = a_np[q];
  }
  const int wid = tid >> 5, lane = tid & 31;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double t = v[k];
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[wid * 64 + k] = t;
  }
  __syncthreads();
  __shared__ double s_tot[64];
  if (tid < NV) {
    double t = 0;
    for (int w = 0; w < kGT / 32; w++) t += red[w * 64 + tid];
    s_tot[tid] = t;
  }
  __syncthreads();
  if (tid == 0) {
    const double *tot = s_tot;
    const double ff = P.final_factor, eps = 1e-15;
    double out[kEccLen];
    for (int k = 0; k < kEccLen; k++) out[k] = 0.0;
    double dn = tot[0];
    for (int n = 1; n < 10; n++) {
      double *o = out + 5 * (n - 1);
      o[4] = (tot[n] * ff) / (dn * ff);
      if (n >= LO && n <= HI && n >= from && n <= to) {
        int q = n - LO;
        o[0] = -(tot[11 + 5 * q] * ff) / (tot[10] * ff + eps);
        o[1] = -(tot[12 + 5 * q] * ff) / (tot[10] * ff + eps);
        o[2] = -(tot[13 + 5 * q] * ff) / (tot[15 + 5 * q] * ff + eps);
        o[3] = -(tot[14 + 5 * q] * ff) / (tot[15 + 5 * q] * ff + eps);
      }
    }
    out[45] = (double)(rec.npart1 + rec.npart2);
    out[46] = (double)rec.ncoll;
    out[47] = xc_sum[0] * ff * P.dx * P.dy;
    out[48] = rec.b;
    for (int k = 0; k < kEccLen; k++) ecc_out[k] = out[k];
  }
  __syncthreads();
}

template <int LO, int HI>
__global__ void __launch_bounds__(kGT) k_grid(DevParams P, int n_events, const EventRec *recs, const Source *srcs,
                                              float *out_rho, float *out_ta, float *out_tb, float *scratch,
                                              double *out_ecc, int *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridLayout L = grid_layout(P.nx, P.ny, P.splat_mw);
  float *acc = reinterpret_cast<float *>(smem + L.off_acc);
  int *list = reinterpret_cast<int *>(smem + L.off_list);
  GroupSrc *grp = reinterpret_cast<GroupSrc *>(smem + L.off_grp);
  float *eyb = reinterpret_cast<float *>(smem + L.off_ey);
  float *xg = reinterpret_cast<float *>(smem + L.off_xg);
  float *yg = reinterpret_cast<float *>(smem + L.off_yg);
  double *red = reinterpret_cast<double *>(smem + L.off_red);
  __shared__ int s_cnt, s_status;
  __shared__ double s_cm[3];

  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int nx = P.nx, ny = P.ny, nyp = L.nyp, mw = L.mw;
  const float inv2w2 = (float)(1.0 / (2.0 * P.w2));
  const float lim = (float)(25.0 * P.w2), lim_lo = lim * (1.f - 1e-4f), lim_hi = lim * (1.f + 1e-4f);
  const float dsq = (float)P.dsq, dsq_lo = dsq * (1.f - 1e-4f), dsq_hi = dsq * (1.f + 1e-4f);
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
    double cm0 = 0, cm1 = 0, cm2 = 0;
    __syncthreads();

    for (int r0 = 0; r0 < nx; r0 += kR) {
      const int rows = min(kR, nx - r0);
      const bool active = r0 + rows > rec.imin && r0 < rec.imax;
      if (active) {
        for (int k = tid; k < 3 * kR * nyp; k += kGT) acc[k] = 0.f;
        __syncthreads();
        for (int c0 = 0; c0 < rec.nsrc; c0 += kGT) {
          // compact the sources of this chunk that reach the strip
          int k = c0 + tid;
          bool hit = false;
          if (k < rec.nsrc) {
            const Source &s = S[k];
            hit = s.xl < r0 + rows && s.xr > r0 && s.yr > s.yl && (s.kind & 15) != 3;
          }
          unsigned bal = __ballot_sync(0xffffffffu, hit);
          if (lane == 0) list[kGT - 1 - wid] = __popc(bal);
          __syncthreads();
          int off = 0, tot = 0;
          for (int q = 0; q < kGT / 32; q++) {
            int cq = list[kGT - 1 - q];
            off += q < wid ? cq : 0;
            tot += cq;
          }
          __syncthreads();
          if (hit) list[off + __popc(bal & ((1u << lane) - 1u))] = k;
          __syncthreads();
          for (int g0 = 0; g0 < tot; g0 += kGS) {
            const int gn = min(kGS, tot - g0);
            // group source descriptors and column factors
            for (int t = tid; t < gn; t += kGT) {
              const Source &s = S[list[g0 + t]];
              GroupSrc g;
              g.x = s.x; g.y = s.y; g.xf = (float)s.x; g.yf = (float)s.y; g.weight = s.weight;
              g.xl = s.xl; g.xr = s.xr; g.yl = s.yl; g.yr = s.yr; g.kind = s.kind; g.plane = s.plane;
              grp[t] = g;
            }
            __syncthreads();
            for (int t = tid; t < gn * mw; t += kGT) {
              int q = t / mw, c = t % mw;
              const GroupSrc &g = grp[q];
              int j = g.yl + c;
              float v = 0.f;
              if (j < g.yr) {
                float dy = yg[j] - g.yf;
                v = (g.kind & 16) ? 1.f : __expf(-dy * dy * inv2w2);
              }
              eyb[q * mw + c] = v;
            }
            __syncthreads();
            // accumulation: warp wid owns row r0 + wid
            const int i = r0 + wid;
            if (wid < rows) {
              const float xgi = xg[i];
              for (int q = 0; q < gn; q++) {
                const GroupSrc &g = grp[q];
                if (i < g.xl || i >= g.xr) continue;
                const float dx = xgi - g.xf;
                const float dx2 = dx * dx;
                const bool disk = g.kind & 16;
                const float exw = disk ? g.weight : g.weight * __expf(-dx2 * inv2w2);
                const float lo = disk ? dsq_lo : lim_lo, hi = disk ? dsq_hi : lim_hi;
                float *arow = acc + ((size_t)g.plane * kR + wid) * nyp;
                for (int j = g.yl + lane; j < g.yr; j += 32) {
                  float dy = yg[j] - g.yf;
                  float dc = fmaf(dy, dy, dx2);
                  bool in = dc < lo;
                  if (!in && dc <= hi) in = cell_in_exact(P, g, i, j);
                  if (in) arow[j] += exw * eyb[q * mw + (j - g.yl)];
                }
              }
            }
            __syncthreads();
          }
        }
      }
      // post-op per cell, outputs and centre-of-mass sums
      float s0 = 0.f, s1 = 0.f, s2 = 0.f;
      for (int c = tid; c < rows * ny; c += kGT) {
        const int rr = c / ny, j = c % ny, i = r0 + rr;
        float v = 0.f, t1 = 0.f, t2 = 0.f;
        if (active) {
          float a0 = acc[(0 * kR + rr) * nyp + j];
          t1 = acc[(1 * kR + rr) * nyp + j];
          t2 = acc[(2 * kR + rr) * nyp + j];
          if (model == 5) v = a0;
          else if (model == 7) v = sqrtf(a0 * t1);
          else if (model == 1) {
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
          if (model == 7) t1 = 0.f, t2 = 0.f;   // planes hold rho_A, rho_B, not T_A, T_B
        }
        rho[(size_t)i * ny + j] = v;
        if (ta) ta[(size_t)i * ny + j] = model == 7 ? 0.f : t1;
        if (tb) tb[(size_t)i * ny + j] = model == 7 ? 0.f : t2;
        s0 += v;
        s1 += xg[i] * v;
        s2 += yg[j] * v;
      }
      cm0 += s0; cm1 += s1; cm2 += s2;
      __syncthreads();
    }
    // ---- centre of mass (FP64 block sums)
    for (int o = 16; o; o >>= 1) {
      cm0 += __shfl_xor_sync(0xffffffffu, cm0, o);
      cm1 += __shfl_xor_sync(0xffffffffu, cm1, o);
      cm2 += __shfl_xor_sync(0xffffffffu, cm2, o);
    }
    if (lane == 0) { red[wid * 3] = cm0; red[wid * 3 + 1] = cm1; red[wid * 3 + 2] = cm2; }
    __syncthreads();
    if (tid == 0) {
      double a = 0, b = 0, c = 0;
      for (int w = 0; w < kGT / 32; w++) { a += red[w * 3]; b += red[w * 3 + 1]; c += red[w * 3 + 2]; }
      s_cm[0] = a; s_cm[1] = b / a; s_cm[2] = c / a;
      if (!(a * P.dx * P.dy >= 1e-15) && s_status == 0) s_status = 5;   // MCnucl.cpp:812-816
    }
    __syncthreads();
    double xcs[3] = {s_cm[0], s_cm[1], s_cm[2]};
    float *xo = xg + nx;
    float *yo = yg + nyp;
    for (int i = tid; i < nx; i += kGT) xo[i] = (float)((P.xmin + i * P.dx) - xcs[1]);
    for (int j = tid; j < ny; j += kGT) yo[j] = (float)((P.ymin + j * P.dy) - xcs[2]);
    __syncthreads();
    moments<LO, HI>(P, rec, S, rho, reinterpret_cast<uint32_t *>(acc), xo, yo, red, xcs,
                    out_ecc + (size_t)e * kEccLen);
    if (tid == 0 && status) status[e] = s_status;
    __syncthreads();
  }
}

size_t grid_smem(const DevParams &P) { return grid_layout(P.nx, P.ny, P.splat_mw).total; }

cudaError_t launch_grid(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs, float *out_rho,
                        float *out_ta, float *out_tb, float *scratch, double *out_ecc, int *status, int grid,
                        cudaStream_t st) {
  size_t smem = grid_layout(P.nx, P.ny, P.splat_mw).total;
  const bool narrow = P.ecc_from >= 2 && P.ecc_to <= 5;
  auto kern = narrow ? k_grid<2, 5> : k_grid<1, 9>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kGT, smem, st>>>(P, n_events, recs, srcs, out_rho, out_ta, out_tb, scratch, out_ecc, status);
  return cudaGetLastError();
}

}  // namespace smc
