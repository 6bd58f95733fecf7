// Adjoint of the MC-Glauber event: gradients of
//     L = sum_e [ gE[e][0] |eps_2(e)| + gE[e][1] |eps_3(e)| + sum_c gG[e][c] rho_e(c) ]
// with respect to the nucleon width w, the mixing parameter alpha and the
// Woods-Saxon R and a (through the sources' position tangents), one CTA per
// event.  No reference counterpart (the reference computes no
// derivatives); the forward quantities follow
//   rho = (1-a)/2 WN + a BC                     src/MCnucl.cpp:688-779
//   eps_n (r^n weighting about the centre of mass, hot-spot region)
//                                               src/MakeDensity.cpp:2244-2511
// The windows, the per-cell cuts, the participant set and the hot-spot
// region are held fixed (they are piecewise constant in the parameters), so
// the gradient is that of the smooth part:
//   rho(c) = sum_s W_s e_s(c),  e_s(c) = exp(-r^2/2w^2) on s's included cells,
//   W = peak (1-a)/2 (participants), peak a (binary collisions), peak = 1/2 pi w^2
//   d rho(c)/d a = sum_s (dW_s/da) e_s(c)
//   d rho(c)/d w = sum_s W_s e_s(c) (r^2/w^3 - 2/w)
//   d rho(c)/d x_s = W_s e_s(c) (x_c - x_s)/w^2   (likewise y)
// Reverse mode: lambda(c) = dL/d rho(c) (including the dependence of the
// centre of mass on rho) is formed on the event's bounding box; then each
// (source, row) pair recomputes its Gaussians (nothing is stored from the
// forward pass) and contracts them with lambda.
#include "grid_common.cuh"
#include "smc_kernels.h"

namespace smc {

constexpr int kAT = 256;
constexpr int kAW = kAT / 32;

struct Cplx {
  float re, im;
};
__device__ __forceinline__ Cplx cmul(Cplx a, Cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// block sum of nv FP32 values per thread into double totals (double-float
// warp reductions)
template <int NV>
__device__ __forceinline__ void block_sums(const float (&v)[NV], float2 *red, double *out) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    DF t = df_warp_sum(DF{v[k], 0.f});
    if (lane == 0) red[wid * 64 + k] = make_float2(t.hi, t.lo);
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double t = 0;
    for (int w = 0; w < kAW; w++) t += (double)red[w * 64 + threadIdx.x].x + (double)red[w * 64 + threadIdx.x].y;
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// shared memory: hot-spot mask [nx][ceil(ny/32)] words, cell coordinates
// xg [nx], yg [ny rounded up to 32], then the reduction slots (16-byte aligned)
__host__ __device__ inline size_t red_offset(int nx, int ny) {
  const size_t nyp = (ny + 31) / 32 * 32, nw = (ny + 31) / 32;
  // mask, xg / yg, then xo / yo (the coordinates about the event's centre of mass)
  const size_t b = sizeof(uint32_t) * (size_t)nx * nw + 2 * sizeof(float) * (nx + nyp);
  return (b + 15) / 16 * 16;
}

__global__ void __launch_bounds__(kAT) k_adjoint(DevParams P, int n_events, const EventRec *recs, const Source *srcs,
                                                 const float4 *src_tan, const float *rho_ev, const float *g_grid, const double *g_eps,
                                                 float *lam_scratch, double *dtheta, EventQueue q) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nx = P.nx, ny = P.ny, nw = (ny + 31) / 32;
  uint32_t *mask = reinterpret_cast<uint32_t *>(smem);
  float *xg = reinterpret_cast<float *>(smem + sizeof(uint32_t) * (size_t)nx * nw);
  float *yg = xg + nx;
  float *xo = yg + (ny + 31) / 32 * 32, *yo = xo + nx;
  float2 *red = reinterpret_cast<float2 *>(smem + red_offset(nx, ny));
  __shared__ double s_tot[32];
  __shared__ double s_coef[8];
  const int tid = threadIdx.x;
  const double w = P.width;
  const float inv2w2 = (float)(1.0 / (2.0 * P.w2));
  const float lim = (float)(25.0 * P.w2), band_g = cut_band(P, 25.0 * P.w2);
  const float lim_lo = lim * (1.f - band_g), lim_hi = lim * (1.f + band_g);
  const float inv_dy = (float)(1.0 / P.dy), ymin_f = (float)P.ymin;
  const int hmax = P.splat_mw;
  for (int i = tid; i < nx; i += kAT) xg[i] = (float)(P.xmin + i * P.dx);
  for (int j = tid; j < ny; j += kAT) yg[j] = (float)(P.ymin + j * P.dy);
  float *lam = lam_scratch + (size_t)blockIdx.x * nx * ny;

  __shared__ int s_k;
  for (int kq = queue_first(q, &s_k); kq < n_events; kq = queue_next(q, kq, &s_k)) {
    const int e = queue_event(q, kq);
    const EventRec rec = recs[e];
    const Source *S = srcs + (size_t)e * P.max_src;
    const float *rho = rho_ev + (size_t)e * nx * ny;
    const float *gg = g_grid ? g_grid + (size_t)e * nx * ny : nullptr;
    const int i0 = rec.imin, i1 = rec.imax, j0 = rec.jmin, j1 = rec.jmax;
    const int bw = j1 > j0 ? j1 - j0 : 0, ncell = i1 > i0 ? (i1 - i0) * bw : 0;
    hotspot_mask<kAT>(P, rec, S, mask);
    // ---- centre of mass (all cells)
    {
      float v[3] = {0.f, 0.f, 0.f};
      KSum a, b, c;
      for (int k = tid; k < ncell; k += kAT) {
        const int i = i0 + k / bw, j = j0 + k % bw;
        const float d = rho[(size_t)i * ny + j];
        a.add(d);
        b.add(xg[i] * d);
        c.add(yg[j] * d);
      }
      v[0] = a.s - a.c; v[1] = b.s - b.c; v[2] = c.s - c.c;
      block_sums<3>(v, red, s_tot);
    }
    const double tot = s_tot[0], xc = s_tot[1] / tot, yc = s_tot[2] / tot;
    const float xcf = (float)xc, ycf = (float)yc;
    // the box's coordinates about the centre of mass, each rounded once from FP64
    for (int i = i0 + tid; i < i1; i += kAT) xo[i] = (float)((P.xmin + i * P.dx) - xc);
    for (int j = j0 + tid; j < j1; j += kAT) yo[j] = (float)((P.ymin + j * P.dy) - yc);
    __syncthreads();
    // ---- masked moments of orders 2 and 3: Z = sum z^n rho, D = sum |z|^n rho,
    // U = sum n z^(n-1) rho, V = sum n |z|^(n-2) z rho (z about the centre of mass)
    {
      float v[14];
#pragma unroll
      for (int k = 0; k < 14; k++) v[k] = 0.f;
      for (int k = tid; k < ncell; k += kAT) {
        const int i = i0 + k / bw, j = j0 + k % bw;
        if (!((mask[i * nw + (j >> 5)] >> (j & 31)) & 1u)) continue;
        const float d = rho[(size_t)i * ny + j];
        if (d == 0.f) continue;
        const Cplx z{xo[i], yo[j]};
        const float r2 = z.re * z.re + z.im * z.im, r = sqrtf(r2);
        const Cplx z2 = cmul(z, z), z3 = cmul(z2, z);
        // order 2
        v[0] += z2.re * d; v[1] += z2.im * d; v[2] += r2 * d;
        v[3] += 2.f * z.re * d; v[4] += 2.f * z.im * d;
        v[5] += 2.f * z.re * d; v[6] += 2.f * z.im * d;
        // order 3
        v[7] += z3.re * d; v[8] += z3.im * d; v[9] += r2 * r * d;
        v[10] += 3.f * z2.re * d; v[11] += 3.f * z2.im * d;
        v[12] += 3.f * r * z.re * d; v[13] += 3.f * r * z.im * d;
      }
      block_sums<14>(v, red, s_tot);
    }
    if (tid == 0) {
      // coefficients of lambda(c): per order A (masked Re(conj Z z^n)), B
      // (masked |z|^n), and the centre-of-mass terms Cx, Cy / tot
      double cx = 0, cy = 0;
      for (int q = 0; q < 2; q++) {
        const double *t = s_tot + 7 * q;
        const double zr = t[0], zi = t[1], dd = t[2] + 1e-15, az = sqrt(zr * zr + zi * zi);
        const double g = g_eps ? g_eps[2 * (size_t)e + q] : 0.0;
        const double A = az > 0 ? g / (az * dd) : 0.0, B = -g * az / (dd * dd);
        s_coef[2 * q] = A;
        s_coef[2 * q + 1] = B;
        // d|eps|/dx_cm = A Re(conj Z dZ/dx_cm) + B dD/dx_cm with dZ/dx_cm = -U,
        // dZ/dy_cm = -i U, dD/dx_cm = -Re V, dD/dy_cm = -Im V
        const double ur = t[3], ui = t[4], vr = t[5], vi = t[6];
        cx += A * (-(zr * ur + zi * ui)) + B * (-vr);
        cy += A * (-(zr * (-ui) + zi * ur)) + B * (-vi);
      }
      s_coef[4] = cx / tot;
      s_coef[5] = cy / tot;
      s_coef[6] = s_tot[0]; s_coef[7] = s_tot[1];   // Z_2 (re, im)
    }
    __syncthreads();
    // ---- lambda on the bounding box
    {
      const double A2 = s_coef[0], B2 = s_coef[1], A3 = s_coef[2], B3 = s_coef[3], Cx = s_coef[4], Cy = s_coef[5];
      const float z2r = (float)s_coef[6], z2i = (float)s_coef[7];
      const float z3r = (float)s_tot[7], z3i = (float)s_tot[8];
      const float cxf = (float)Cx, cyf = (float)Cy, a2 = (float)A2, b2 = (float)B2, a3 = (float)A3, b3 = (float)B3;
      // a warp per row of the box, lanes over its columns (each cell on its own)
      for (int i = i0 + (tid >> 5); i < i1; i += kAW)
        for (int j = j0 + (tid & 31); j < j1; j += 32) {
          const float x = xg[i] - xcf, y = yg[j] - ycf;
          float l = fmaf(cxf, x, cyf * y);
          if ((mask[i * nw + (j >> 5)] >> (j & 31)) & 1u) {
            const Cplx z{xo[i], yo[j]};
            const float r2 = z.re * z.re + z.im * z.im, r = sqrtf(r2);
            const Cplx zz2 = cmul(z, z), zz3 = cmul(zz2, z);
            l += a2 * (z2r * zz2.re + z2i * zz2.im) + b2 * r2;
            l += a3 * (z3r * zz3.re + z3i * zz3.im) + b3 * r2 * r;
          }
          if (gg) l += gg[(size_t)i * ny + j];
          lam[(size_t)i * ny + j] = l;
        }
    }
    __syncthreads();
    // ---- contraction: one (source, row) pair per thread, Gaussians recomputed.
    // With position tangents t_s = d(x_s, y_s)/d(R, a):
    //   dL/dR += (W/w^2) sum_c lambda e (x_c - x_s, y_c - y_s) . t_s(R)
    float dw = 0.f, da = 0.f, dR = 0.f, dA = 0.f;
    const float4 *T = src_tan ? src_tan + (size_t)e * P.max_src : nullptr;
    const float inv_w2 = (float)(1.0 / P.w2);
    {
      const float peak = (float)P.peak, alpha = (float)P.alpha;
      const int npair = rec.nsrc * hmax;
      for (int q = tid; q < npair; q += kAT) {
        const int k = q / hmax;
        const Source &s = S[k];
        const int kind = s.kind & 15;
        if (kind >= 3 || kind == SRC_THICK || s.xr <= s.xl || s.yr <= s.yl) continue;
        const int i = s.xl + (q - k * hmax);
        if (i >= s.xr) continue;
        const float xf = (float)s.x, yf = (float)s.y;
        const float dx = xg[i] - xf, dx2 = dx * dx;
        int ja, jb;
        cut_interval(P, &s.x, s.kind, yf, i, dx2, lim_lo, lim_hi, yg, inv_dy, ymin_f, s.yl, s.yr, ja, jb);
        if (ja >= jb) continue;
        const float ex = __expf(-dx2 * inv2w2);
        float l0 = 0.f, lr = 0.f, ly = 0.f;
        const float *lrow = lam + (size_t)i * ny;
        for (int j = ja; j < jb; j++) {
          const float dy = yg[j] - yf, dy2 = dy * dy;
          const float t = lrow[j] * __expf(-dy2 * inv2w2);
          l0 += t;
          lr += t * dy2;
          ly += t * dy;
        }
        l0 *= ex;
        ly *= ex;
        lr = ex * lr + dx2 * l0;   // sum lambda e (dx^2 + dy^2)
        const float W = s.weight;
        // W = f peak (1-a)/2 for participants, f peak (a + (1-a) aw) for
        // binary collisions (aw in {0, 1, 2}, nonzero with sub_model 2; f the
        // multiplicity weight, held fixed, 1 without fluctuations)
        float dWda = alpha < 1.f ? -W / (1.f - alpha) : -0.5f * peak;
        if (kind == SRC_COLL) {
          const float aw = (float)((s.kind >> SRC_AW_SHIFT) & 3);
          dWda = W * (1.f - aw) / (alpha + (1.f - alpha) * aw);
        }
        dw += W * (lr / (float)(w * w * w) - 2.f * l0 / (float)w);
        da += dWda * l0;
        if (T) {
          const float4 t = T[k];
          const float c = W * inv_w2, lx = dx * l0;
          dR += c * (lx * t.x + ly * t.y);
          dA += c * (lx * t.z + ly * t.w);
        }
      }
    }
    {
      float v[4] = {dw, da, dR, dA};
      block_sums<4>(v, red, s_tot);
    }
    if (tid == 0)
      for (int q = 0; q < 4; q++) dtheta[4 * (size_t)e + q] = s_tot[q];
    __syncthreads();
  }
}

size_t adjoint_smem(const DevParams &P) { return red_offset(P.nx, P.ny) + sizeof(float2) * kAW * 64; }

int adjoint_blocks_per_sm(const DevParams &P) {
  const size_t smem = adjoint_smem(P);
  if (cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
  int nb = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_adjoint, kAT, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

cudaError_t launch_adjoint(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs,
                           const float4 *src_tan, const float *rho_ev, const float *g_grid, const double *g_eps,
                           float *lam_scratch, double *dtheta, int grid, cudaStream_t st, const int *order,
                           int *ticket) {
  const size_t smem = adjoint_smem(P);
  cudaError_t e = cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (ticket) {
    e = cudaMemsetAsync(ticket, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
  }
  k_adjoint<<<grid, kAT, smem, st>>>(P, n_events, recs, srcs, src_tan, rho_ev, g_grid, g_eps, lam_scratch, dtheta,
                                     EventQueue{order, ticket});
  return cudaGetLastError();
}

}  // namespace smc
