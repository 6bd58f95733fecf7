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
// it.  Each lane then owns one column of the strip (a warp 32 adjacent
// columns), holds the strip's kR rows of one plane in registers and adds
// the group's sources that reach its columns (a bit mask per 32-column
// block and plane) in order: the column factor exp(-dy^2/2w^2) once per
// source, then one predicated FMA per row inside that row's interval.  No
// atomics: every cell has one owner, so the sums are deterministic.
// All reductions run in FP32 pairs (double-float): FP64 arithmetic is rare
// on this part and used only for the per-event totals.
#include "grid_common.cuh"
#include "smc_kernels.h"

namespace smc {

constexpr int kGT = 256;            // threads per CTA
constexpr int kWarps = kGT / 32;
constexpr int kR = 8;               // rows per strip (held in registers by the accumulating lanes)
constexpr int kGS = 64;             // sources per group
constexpr int kGW = kGS / 32;       // 32-bit words of a group's source mask
static_assert(kGS % 32 == 0, "source masks are whole words");
constexpr int kRU = kR;             // rows of a work unit
static_assert(kRU % 4 == 0, "units are read four rows at a time");

// (source, row) pairs of a strip, structure of arrays [kGS][kR]: the row
// factor weight * exp(-dx^2 / 2w^2), the first included column and the
// number of included columns (0: the source misses the row)
struct GridLayout {
  int nyp, mw, np;
  size_t off_acc, off_list, off_grp, off_exw, off_ja, off_len, off_xg, off_yg, off_red, total;
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
  o = (o + 15) / 16 * 16;
  L.off_exw = o; o += sizeof(float) * kGS * kR;
  L.off_ja = o; o += sizeof(int) * kGS * kR;
  L.off_len = o; o += sizeof(int) * kGS * kR;
  o = (o + 15) / 16 * 16;
  L.off_xg = o; o += sizeof(float) * 2 * nx;   // grid x, then x - x_cm
  L.off_yg = o; o += sizeof(float) * 2 * L.nyp;
  o = (o + 15) / 16 * 16;
  // the reduction slots are used after the strips (centre of mass, moments):
  // inside the accumulator region after the mask when they fit there
  const size_t red_bytes = sizeof(float2) * kWarps * 64, acc_bytes = sizeof(float) * np * kR * L.nyp;
  const size_t red_in = (mask_bytes + 15) / 16 * 16;
  if (red_in + red_bytes <= acc_bytes) {
    L.off_red = L.off_acc + red_in;
  } else {
    L.off_red = o;
    o += red_bytes;
  }
  L.total = o;
  return L;
}

// column steps of 32 cells whose MC-KLN fix-up marks one 64-bit word holds
constexpr int kPendSteps = 32;

// The MC-KLN cells of row i, columns s0 + 32 k + lane, that post_cell left
// undecided (pend: two bits per step k, the planes to redo), finished by the
// whole warp in step and lane order: the flagged thickness sums redone in
// FP64 (thickness_fp64), then each cell's owner lane writes its outputs and
// adds it to its centre-of-mass sums (so the sums keep one deterministic
// order).  t_a, t_b: the strip's T_A and T_B rows.  The sums go in and come
// back by value (their addresses are never taken, so they stay in registers
// in the caller's loops).
template <bool NBD>
static __device__ __noinline__ CmSums kln_finish_row(const DevParams &P, const EventRec &rec, const Source *S,
                                                     const float *t_a, const float *t_b, int i, int s0, uint64_t pend,
                                                     float *rho, float *ta, float *tb, float xi, const float *yg,
                                                     CmSums cs, int *s_status) {
  const int lane = threadIdx.x & 31, ny = P.ny;
  for (int k = 0; k < kPendSteps; k++) {
    const unsigned need = (unsigned)(pend >> (2 * k)) & 3u;
    unsigned m = __ballot_sync(0xffffffffu, need != 0);
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1u;
      const int j = s0 + 32 * k + src;
      const unsigned nd = __shfl_sync(0xffffffffu, need, src);
      // the FP32 values as post_cell took them (below kln_tzero: zero)
      const float a0 = t_a[j] < P.kln_tzero ? 0.f : t_a[j], a1 = t_b[j] < P.kln_tzero ? 0.f : t_b[j];
      const double da = (nd & 1u) ? thickness_fp64(P, S, rec.nsplat - rec.npart1 - rec.npart2, rec.npart1, 0, i, j)
                                  : (double)a0;
      const double db = (nd & 2u) ? thickness_fp64(P, S, rec.nsplat - rec.npart2, rec.npart2, 1, i, j) : (double)a1;
      if (lane == src) {
        float v, t1, t2;
        if (kln_cell_fp64(P, da, db, v, t1, t2) == CELL_TABLE) *s_status = 4;
        if (NBD) {
          cs.pre.add(v);
          v = nbd_cell(P, rec.ev, (uint32_t)(i * ny + j), v, t1, t2);
        }
        rho[(size_t)i * ny + j] = v;
        if (ta) ta[(size_t)i * ny + j] = t1;
        if (tb) tb[(size_t)i * ny + j] = t2;
        if (v != 0.f) {
          cs.c0.add(v);
          cs.c1.add(xi * v);
          cs.c2.add(yg[j] * v);
        }
      }
    }
  }
  return cs;
}

// NBD: the per-cell negative-binomial fluctuations (a separate instance, so
// that the common case carries none of their registers)
template <int LO, int HI, bool NBD>
// five CTAs per SM (51 registers per thread, shared memory for five 8-row strips):
// latency-bound work wants resident warps more than registers
__global__ void __launch_bounds__(kGT, 5) k_grid(DevParams P, int n_events, const EventRec *recs, const Source *srcs,
                                              float *out_rho, float *out_ta, float *out_tb, float *scratch,
                                              double *out_ecc, int *status, EventQueue q) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridLayout L = grid_layout(P.nx, P.ny, P.splat_mw, P.n_planes);
  float *acc = reinterpret_cast<float *>(smem + L.off_acc);
  int *list = reinterpret_cast<int *>(smem + L.off_list);
  GroupSrc *grp = reinterpret_cast<GroupSrc *>(smem + L.off_grp);
  float *p_exw = reinterpret_cast<float *>(smem + L.off_exw);
  int *p_ja = reinterpret_cast<int *>(smem + L.off_ja);
  int *p_len = reinterpret_cast<int *>(smem + L.off_len);
  float *xg = reinterpret_cast<float *>(smem + L.off_xg);
  float *yg = reinterpret_cast<float *>(smem + L.off_yg);
  float2 *red = reinterpret_cast<float2 *>(smem + L.off_red);
  __shared__ int s_status;
  __shared__ int s_wcnt[kWarps];
  __shared__ double s_cm[3];

  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int nx = P.nx, ny = P.ny, nyp = L.nyp, np = L.np;
  // Gaussian factors 2^(-d^2 c) of grid distances d (gauss_grid)
  const float cx = (float)(P.dx * P.dx * 1.4426950408889634 / (2.0 * P.w2));
  const float cy = (float)(P.dy * P.dy * 1.4426950408889634 / (2.0 * P.w2));
  const float lim = (float)(25.0 * P.w2), band_g = cut_band(P, 25.0 * P.w2);
  const float lim_lo = lim * (1.f - band_g), lim_hi = lim * (1.f + band_g);
  const float dsq = (float)P.dsq, band_d = cut_band(P, P.dsq);
  const float dsq_lo = dsq * (1.f - band_d), dsq_hi = dsq * (1.f + band_d);
  const float inv_dy = (float)(1.0 / P.dy), ymin_f = (float)P.ymin;

  for (int i = tid; i < nx; i += kGT) xg[i] = (float)(P.xmin + i * P.dx);
  for (int j = tid; j < nyp; j += kGT) yg[j] = j < ny ? (float)(P.ymin + j * P.dy) : 0.f;

  __shared__ int s_k;
  for (int k = queue_first(q, &s_k); k < n_events; k = queue_next(q, k, &s_k)) {
    const int e = queue_event(q, k);
    const EventRec rec = recs[e];
    const Source *S = srcs + (size_t)e * P.max_src;
    float *rho = out_rho ? out_rho + (size_t)e * nx * ny : scratch + (size_t)blockIdx.x * nx * ny;
    float *ta = out_ta ? out_ta + (size_t)e * nx * ny : nullptr;
    float *tb = out_tb ? out_tb + (size_t)e * nx * ny : nullptr;
    if (tid == 0) s_status = rec.status;
    KSum cm0, cm1, cm2, pre;   // pre: the density before NBD fluctuations (the zero-dN/dy test)
    const bool full = out_rho || ta || tb;
    const float kband = kln_event_band(P, rec);
    // the 32-column blocks of the event's window box: the accumulators
    // outside them are never written or read
    const int jb0 = rec.jmin >> 5, nunits = rec.jmax > rec.jmin ? (((rec.jmax + 31) >> 5) - jb0) * np : 0;
    __syncthreads();

    for (int r0 = 0; r0 < nx; r0 += kR) {
      const int rows = min(kR, nx - r0);
      const bool active = r0 + rows > rec.imin && r0 < rec.imax;
      // fresh: no group accumulated yet (the accumulators are not read back,
      // and a strip no source reaches has no valid accumulators)
      bool fresh = true;
      if (active) {
        for (int c0 = 0; c0 < rec.nsplat; c0 += kGT) {   // the splat sources lead the records
          // compact the sources of this chunk that reach the strip
          int k = c0 + tid;
          bool hit = false;
          if (k < rec.nsplat) {
            const Source &s = S[k];
            hit = s.xl < r0 + rows && s.xr > r0 && s.yr > s.yl && (s.kind & 15) < 3;   // kinds >= 3: no splat
          }
          unsigned bal = __ballot_sync(0xffffffffu, hit);
          if (lane == 0) s_wcnt[wid] = __popc(bal);
          __syncthreads();
          int off = 0, tot = 0;
          for (int q = 0; q < kWarps; q++) {
            int cq = s_wcnt[q];
            off += q < wid ? cq : 0;
            tot += cq;
          }
          if (hit) list[off + __popc(bal & ((1u << lane) - 1u))] = k;
          __syncthreads();
          for (int g0 = 0; g0 < tot; g0 += kGS) {
            const int gn = min(kGS, tot - g0);
            // row factors and included column intervals, one per (source,
            // row); the row-0 thread of a source also stores it for the
            // accumulating warps
            for (int t = tid; t < gn; t += kGT) {
              const Source &s = S[list[g0 + t]];
              GroupSrc g;
              g.x = s.x; g.y = s.y; g.xf = (float)s.x; g.yf = (float)s.y; g.weight = s.weight;
              g.gi0 = s.gi0; g.gfx = s.gfx; g.gj0 = s.gj0; g.gfy = s.gfy;
              g.xl = s.xl; g.xr = s.xr; g.yl = s.yl; g.yr = s.yr;
              g.kind = s.kind; g.plane = s.plane;
              grp[t] = g;
            }
            __syncthreads();
            for (int t = tid; t < gn * kR; t += kGT) {
              const int q = t / kR, r = t - q * kR;
              const GroupSrc g = grp[q];
              const int i = r0 + r;
              float exw = 0.f;
              int ja = 0, len = 0;
              if (r < rows && i >= g.xl && i < g.xr) {
                const bool disk = g.kind & 16;
                const float dx = xg[i] - g.xf, dx2 = dx * dx;
                exw = disk ? g.weight : g.weight * gauss_grid((float)i, g.gi0, g.gfx, cx);
                int jb;
                row_interval(P, g, i, dx2, disk ? dsq_lo : lim_lo, disk ? dsq_hi : lim_hi, yg, inv_dy, ymin_f, ja,
                             jb);
                len = max(jb - ja, 0);
              }
              p_exw[t] = exw;
              p_ja[t] = ja;
              p_len[t] = len;
            }
            __syncthreads();
            // accumulation: lane owns column j of the strip; the work units are
            // (32-column block of the event's box, plane), dealt to the warps
            // round robin so that the busy central blocks and the two planes
            // spread over them; each unit visits only the sources of its
            // plane that reach its block, in order
            for (int u = wid; u < nunits; u += kWarps) {
              const int ub = np == 1 ? u : u / np, pl = u - ub * np;
              const int jb = jb0 + ub, j = jb * 32 + lane;
              const float jf = (float)j;
              // the group's sources whose window reaches this block: lane q
              // of word h tests source 32 h + q
              bool qin[kGW];
#pragma unroll
              for (int h = 0; h < kGW; h++) {
                const int q = h * 32 + lane;
                qin[h] = false;
                if (q < gn) {
                  const GroupSrc &g = grp[q];
                  qin[h] = g.yr > jb * 32 && g.yl < jb * 32 + 32 && g.yr > g.yl && g.plane == pl;
                }
              }
              {
                float *ab = acc + (size_t)pl * kR * nyp + j;
                float a[kRU];
#pragma unroll
                for (int r = 0; r < kRU; r++) a[r] = fresh ? 0.f : ab[r * nyp];
#pragma unroll
                for (int h = 0; h < kGW; h++) {
                  uint32_t m = __ballot_sync(0xffffffffu, qin[h]);
                  while (m) {
                    const int q = h * 32 + __ffs(m) - 1;
                    m &= m - 1u;
                    const GroupSrc &g = grp[q];
                    const float ey = (g.kind & 16) ? 1.f : gauss_grid(jf, g.gj0, g.gfy, cy);
#pragma unroll
                    for (int r4 = 0; r4 < kRU; r4 += 4) {
                      const int o = q * kR + r4;
                      const float4 w4 = *reinterpret_cast<const float4 *>(p_exw + o);
                      const int4 a4 = *reinterpret_cast<const int4 *>(p_ja + o);
                      const int4 l4 = *reinterpret_cast<const int4 *>(p_len + o);
                      if ((unsigned)(j - a4.x) < (unsigned)l4.x) a[r4] += w4.x * ey;
                      if ((unsigned)(j - a4.y) < (unsigned)l4.y) a[r4 + 1] += w4.y * ey;
                      if ((unsigned)(j - a4.z) < (unsigned)l4.z) a[r4 + 2] += w4.z * ey;
                      if ((unsigned)(j - a4.w) < (unsigned)l4.w) a[r4 + 3] += w4.w * ey;
                    }
                  }
                }
#pragma unroll
                for (int r = 0; r < kRU; r++) ab[r * nyp] = a[r];
              }
            }
            fresh = false;
            __syncthreads();
          }
        }
      }
      // post-op per cell, outputs and centre-of-mass sums.  Scratch grids
      // are read back only inside the event's window bounding box, so only
      // that part is written; output grids are written whole.
      if (active || full) {
        const int jlo = full ? 0 : rec.jmin, jhi = full ? ny : rec.jmax;
        for (int rr = wid; rr < rows; rr += kWarps) {
          const int i = r0 + rr;
          // segments of up to 32 column steps: the MC-KLN cells left
          // undecided in FP32 are marked (the planes to redo, two bits per
          // step) and finished by the warp after the segment, outside the
          // per-cell loop
          for (int s0 = jlo; s0 < jhi; s0 += 32 * kPendSteps) {
            const int s1 = min(jhi, s0 + 32 * kPendSteps);
            uint64_t pend = 0;
            // the lane's sums over the segment's cells in FP32 (at most
            // kPendSteps terms), added to the compensated sums after it
            float p0 = 0.f, p2 = 0.f, pp = 0.f;
            for (int j = s0 + lane; j < s1; j += 32) {
              float v = 0.f, t1 = 0.f, t2 = 0.f;
              if (active && !fresh && j >= rec.jmin && j < rec.jmax) {
                const float a0 = acc[rr * nyp + j];
                const float a1 = np > 1 ? acc[(kR + rr) * nyp + j] : 0.f;
                const float a2 = np > 2 ? acc[(2 * kR + rr) * nyp + j] : 0.f;
                const int code = post_cell(P, np, a0, a1, a2, kband, v, t1, t2);
                if (code & CELL_UNDECIDED) {
                  pend |= (uint64_t)((code & (CELL_NEED_A | CELL_NEED_B)) >> 4) << (2 * ((j - s0) >> 5));
                  continue;
                }
                if (code == CELL_TABLE) s_status = 4;
                if (NBD) {
                  pp += v;
                  v = nbd_cell(P, rec.ev, (uint32_t)(i * ny + j), v, t1, t2);
                }
              }
              rho[(size_t)i * ny + j] = v;
              if (ta) ta[(size_t)i * ny + j] = t1;
              if (tb) tb[(size_t)i * ny + j] = t2;
              p0 += v;
              p2 += yg[j] * v;
            }
            cm0.add(p0);
            cm1.add(xg[i] * p0);
            cm2.add(p2);
            if (NBD) pre.add(pp);
            if (P.which_mc_model == 1 && __any_sync(0xffffffffu, pend != 0)) {
              const CmSums cs = kln_finish_row<NBD>(P, rec, S, acc + rr * nyp, acc + (kR + rr) * nyp, i, s0, pend,
                                                    rho, ta, tb, xg[i], yg, CmSums{cm0, cm1, cm2, pre}, &s_status);
              cm0 = cs.c0; cm1 = cs.c1; cm2 = cs.c2; pre = cs.pre;
            }
          }
        }
      }
    }
    __syncthreads();   // the post-op's reads of the strip are done (the reductions reuse its memory)
    // ---- centre of mass
    {
      DF a = df_warp_sum(cm0.df()), b = df_warp_sum(cm1.df()), c = df_warp_sum(cm2.df()), d = df_warp_sum(pre.df());
      if (lane == 0) {
        red[wid * 64] = make_float2(a.hi, a.lo);
        red[wid * 64 + 1] = make_float2(b.hi, b.lo);
        red[wid * 64 + 2] = make_float2(c.hi, c.lo);
        red[wid * 64 + 3] = make_float2(d.hi, d.lo);
      }
      __syncthreads();
      if (tid < 32) {   // lane k < 4 adds sum k (FP64, warp order), lanes 1, 2 divide
        double t = 0;
        if (lane < 4)
          for (int w = 0; w < kWarps; w++) t += (double)red[w * 64 + lane].x + (double)red[w * 64 + lane].y;
        const double sa = __shfl_sync(0xffffffffu, t, 0), sd = __shfl_sync(0xffffffffu, t, 3);
        if (lane == 0) {
          s_cm[0] = sa;
          // MCnucl.cpp:812-816, on the density before the NBD fluctuations (:819)
          if (!((NBD ? sd : sa) * P.dx * P.dy >= 1e-15) && s_status == 0) s_status = 5;
        } else if (lane < 3) {
          s_cm[lane] = t / sa;
        }
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
      moments<LO, HI, kGT>(P, rec, S, rho, reinterpret_cast<uint32_t *>(acc), xo, yo, red, tot0,
                      out_ecc + (size_t)e * kEccLen);
    if (tid == 0 && status) status[e] = s_status;
    __syncthreads();
  }
}

size_t grid_smem(const DevParams &P) { return grid_layout(P.nx, P.ny, P.splat_mw, P.n_planes).total; }

int grid_blocks_per_sm(const DevParams &P) {
  const bool narrow = P.ecc_from >= 2 && P.ecc_to <= 5;
  const void *k = P.nbd ? (narrow ? (const void *)k_grid<2, 5, true> : (const void *)k_grid<1, 9, true>)
                        : (narrow ? (const void *)k_grid<2, 5, false> : (const void *)k_grid<1, 9, false>);
  size_t smem = grid_smem(P);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
  int nb = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kGT, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

cudaError_t launch_grid(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs, float *out_rho,
                        float *out_ta, float *out_tb, float *scratch, double *out_ecc, int *status, int grid,
                        cudaStream_t st, const int *order, int *ticket) {
  size_t smem = grid_smem(P);
  const bool narrow = P.ecc_from >= 2 && P.ecc_to <= 5;
  auto kern = P.nbd ? (narrow ? k_grid<2, 5, true> : k_grid<1, 9, true>)
                    : (narrow ? k_grid<2, 5, false> : k_grid<1, 9, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (ticket) {
    e = cudaMemsetAsync(ticket, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
  }
  kern<<<grid, kGT, smem, st>>>(P, n_events, recs, srcs, out_rho, out_ta, out_tb, scratch, out_ecc, status,
                                EventQueue{order, ticket});
  return cudaGetLastError();
}

}  // namespace smc
