// Stage 2 of the event pipeline on the tensor cores: the Gaussian splat of
// the thickness / density planes as a separable contraction, one event at a
// time per CTA, one CTA per SM (persistent over the batch).
//
// Reference behaviour restated here (the same as k_grid.cu):
//   T_A, T_B (Gaussian nucleons, r <= 5w)     src/MCnucl.cpp:432-478, src/Particle.cpp:122-132
//   Glauber rho = (1-a)/2 WN + a BC            src/MCnucl.cpp:688-779, :822-866
//   sqrt(T_A T_B), MC-KLN table lookup         src/MCnucl.cpp:654-687, :780-811
//   centre of mass, <r^n>, eps_n               src/MakeDensity.cpp:2244-2511
//
// Inside a source's window [xl,xr) x [yl,yr) the reference adds
// w exp(-dx^2/2w^2) exp(-dy^2/2w^2) except at the cells beyond its cut
// (r > 5w, or dc > 25 w^2 for binary collisions).  Without the cut the sum
// over sources is the matrix product
//     plane = Gx diag(w) Gy^T,   Gx[i,s] = exp(-(x_i-x_s)^2/2w^2) [xl_s <= i < xr_s],
//                                Gy[j,s] = exp(-(y_j-y_s)^2/2w^2) [yl_s <= j < yr_s],
// which runs here as tcgen05 MMAs (kind::tf32, M = 128 grid rows, N = 64
// grid columns, K = sources) with FP32 accumulation in TMEM.  Each factor
// is split into TF32 hi + lo parts and the product is the three-term sum
// hi*hi + hi*lo + lo*hi (representation error ~2^-22).  The tensor core's
// FP32 accumulation loses a fraction of an ulp, always downward, at each
// MMA that adds to a cell (measured: a -1.8e-6 relative drift of the cells
// of central Pb+Pb events over ~50 k-steps).  So TMEM only holds the sum of
// one chunk of kKC sources (two k-steps): after each chunk the hi*hi
// accumulator and the separate cross-term accumulator (2^-11 smaller, its
// loss negligible) are added in round-to-nearest FP32 into the tile's
// shared-memory planes.  Chunks alternate between two operand buffers and
// two TMEM accumulator sets, so the next chunk's operands are built while
// the tensor core works on the current one.
//
// The window cells beyond the cut (the corners of the window; values below
// e^-12.5 of the source's peak) are removed on the CUDA cores: before the
// tiles, one thread per (source, row) of the event finds the exact column
// interval of the reference's FP64 test and adds the window cells outside
// it to a per-cell correction grid in 32-bit fixed point (unit 2^-39 of
// the peak height; the CTA's own grid in global memory, L2-resident;
// integer sums do not depend on the order of the atomic adds).  The
// tiles subtract the corrections, so the planes hold the reference's
// sums; exact sums are non-negative, so a rounding residue below zero is
// cleared.  Every cell of a tile has one owner thread (tile row = its TMEM
// lane, one quarter of the columns) that adds the chunk sums and runs the
// post-op, so results do not depend on scheduling.  k_grid_tc writes each
// event's density and centre-of-mass sums; k_moments (many CTAs per SM)
// then reduces the eccentricities.
//
// k_grid_tc uses 16 warps and keeps the event's splat sources in shared
// memory (one CTA per SM by its registers and shared memory).  At most two
// planes (MC-KLN T_A, T_B; sqrt(T_A T_B); Glauber rho) fit.
#include "grid_common.cuh"
#include "smc_kernels.h"
#include "tc_ptx.cuh"

#include <algorithm>

namespace smc {

constexpr int kTT = 512;                 // threads per CTA
constexpr int kTW = kTT / 32;            // warps
constexpr int kTM = 128;                 // tile rows = TMEM lanes = MMA M
constexpr int kTN = 64;                  // tile columns per plane = MMA N
constexpr int kQ = kTN / 4;              // columns owned by one thread
constexpr int kKC = 16;                  // sources per operand chunk (2 MMA k-steps of 8)
constexpr int kSP = kTN + 1;             // staged row pitch in floats
constexpr int kCap = 512;                // splat sources held in shared memory at once
constexpr int kMaxPlanes = 2;
// corner corrections are integers in units of peak * 2^-39: a cell's sum of
// corner values stays below 4e-3 peak (the cut removes values below
// e^-12.5 peak per source; weights are below 2 peaks)
constexpr float kCorrScale = 549755813888.0f;   // 2^39
constexpr uint32_t kOpA = kTM * kKC * 4; // bytes of one A copy (hi or lo)
constexpr uint32_t kOpB = kTN * kKC * 4; // bytes of one B copy
constexpr uint32_t kOpSet = 2 * (kOpA + kOpB);   // one operand buffer: A hi, A lo, B hi, B lo
// K-major, no swizzle: core matrices of 8 rows x 16 bytes (4 TF32 values).
// Cores adjacent in M/N are 128 bytes apart (SBO); cores adjacent in K are
// one full column of cores apart (LBO).  Element (r, k) then sits at byte
// 4 * idx with idx = 32 * core + 4 * (r % 8) + k % 4, core = (k / 4) * (R / 8) + r / 8.
constexpr uint32_t kLboA = kTM * 16, kLboB = kTN * 16, kSbo = 128;
// two accumulator sets (chunks alternate), each hi*hi + cross terms, kTN columns each
constexpr uint32_t kTmemCols = 4 * kTN;
constexpr uint32_t kMaxPolls = 1u << 24; // MMA completion wait limit
constexpr int kErrMmaTimeout = 8;        // per-event status when that limit is hit
constexpr int kPendCapTc = 128;          // undecided MC-KLN cells an event's list holds

// A splat source held in shared memory.
struct CSrc {
  float xf, yf, w;
  float gi0, gfx, gj0, gfy;   // grid cell and fraction of the position (grid_offset)
  int16_t xl, xr, yl, yr, kind, plane;
  int idx;   // index in the event's source array (FP64 position for the exact test)
};

struct TcLayout {
  int nyp;
  size_t off_stage, off_cache, off_list, off_xg, off_yg, off_red, total;
};

// Two operand buffers, the tile's accumulator planes, the source cache;
// the eccentricity mask reuses the first region after the last tile.
__host__ __device__ inline TcLayout tc_layout(int nx, int ny, int np) {
  TcLayout L;
  L.nyp = (ny + 31) / 32 * 32;
  size_t o = 2 * (size_t)kOpSet;
  L.off_stage = o; o += sizeof(float) * (size_t)np * kTM * kSP;
  const size_t mk = sizeof(uint32_t) * (size_t)nx * (L.nyp / 32);
  if (mk > o) o = mk;
  o = (o + 15) / 16 * 16;
  L.off_cache = o; o += sizeof(CSrc) * kCap;
  L.off_list = o; o += sizeof(int16_t) * kCap;
  o = (o + 15) / 16 * 16;
  L.off_xg = o; o += sizeof(float) * 2 * nx;     // grid x, then x - x_cm
  L.off_yg = o; o += sizeof(float) * 2 * L.nyp;
  o = (o + 15) / 16 * 16;
  L.off_red = o; o += sizeof(float2) * kTW * 64;
  L.total = o;
  return L;
}

// Block-wide compaction of up to kTT candidates: indices v with hit set, in
// thread order, appended to list at count (block-uniform; updated).
__device__ __forceinline__ void compact_append(bool hit, int v, int16_t *list, int *wcnt, int &count) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned bal = __ballot_sync(0xffffffffu, hit);
  if (lane == 0) wcnt[wid] = __popc(bal);
  __syncthreads();
  int off = 0, tot = 0;
#pragma unroll
  for (int q = 0; q < kTW; q++) {
    const int c = wcnt[q];
    off += q < wid ? c : 0;
    tot += c;
  }
  if (hit) list[count + off + __popc(bal & ((1u << lane) - 1u))] = (int16_t)v;
  __syncthreads();
  count += tot;
}

__device__ __forceinline__ bool splat_source(const Source &s) {
  return (s.kind & 15) < 3 && s.xr > s.xl && s.yr > s.yl;   // kinds >= 3: no splat
}

__global__ void __launch_bounds__(kTT, 1) k_grid_tc(DevParams P, int n_events, const EventRec *recs,
                                                    const Source *srcs, float *out_rho, float *out_ta,
                                                    float *out_tb, float *rho_ev, int *corr_scratch,
                                                    double *cm_ev, int *status, EventQueue q) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int np = P.n_planes;
  const TcLayout L = tc_layout(P.nx, P.ny, np);
  float *stage = reinterpret_cast<float *>(smem + L.off_stage);
  CSrc *cache = reinterpret_cast<CSrc *>(smem + L.off_cache);
  int16_t *list = reinterpret_cast<int16_t *>(smem + L.off_list);
  float *xg = reinterpret_cast<float *>(smem + L.off_xg);
  float *yg = reinterpret_cast<float *>(smem + L.off_yg);
  float2 *red = reinterpret_cast<float2 *>(smem + L.off_red);
  __shared__ uint64_t s_bar[2];
  __shared__ uint32_t s_tmem;
  __shared__ int s_wcnt[kTW];
  __shared__ int s_status, s_dead, s_ncache;
  // the event's undecided MC-KLN cells, decided together at its end by all
  // warps (a cell that finds the list full is decided at once by its warp)
  __shared__ PendCell s_pend[kPendCapTc];
  __shared__ int s_npend;
  __shared__ double s_cm[3];

  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int nx = P.nx, ny = P.ny;
  // Gaussian factors 2^(-d^2 c) of grid distances d (gauss_grid)
  const float cx = (float)(P.dx * P.dx * 1.4426950408889634 / (2.0 * P.w2));
  const float cy = (float)(P.dy * P.dy * 1.4426950408889634 / (2.0 * P.w2));
  const float lim = (float)(25.0 * P.w2), band_g = cut_band(P, 25.0 * P.w2);
  const float lim_lo = lim * (1.f - band_g), lim_hi = lim * (1.f + band_g);
  const float inv_dy = (float)(1.0 / P.dy), ymin_f = (float)P.ymin;
  const uint32_t idesc = tc::idesc_tf32(kTM, kTN);
  // the cells this thread owns in every tile: row r (TMEM lane r; warp w may
  // read lanes 32 (w % 4) .. +31) and columns kQ*hc .. +kQ-1 of each plane
  const int r_own = tid & (kTM - 1), hc = tid / kTM;
  const uint32_t tm_lanes = (uint32_t)(32 * (wid & 3)) << 16;
  const int hmax = P.splat_mw;                       // rows of a window, at most
  const float corr_unit = (float)P.peak / kCorrScale, inv_corr_unit = kCorrScale / (float)P.peak;

  for (int i = tid; i < nx; i += kTT) xg[i] = (float)(P.xmin + i * P.dx);
  for (int j = tid; j < ny; j += kTT) yg[j] = (float)(P.ymin + j * P.dy);
  if (wid == 0) {
    tc::tmem_alloc(&s_tmem, kTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&s_bar[0], 1);
    tc::mbar_init(&s_bar[1], 1);
    tc::fence_mbar_init();
    s_dead = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  uint32_t phase[2] = {0u, 0u};

  __shared__ int s_k;
  for (int k = queue_first(q, &s_k); k < n_events; k = queue_next(q, k, &s_k)) {
    const int e = queue_event(q, k);
    const EventRec rec = recs[e];
    const Source *S = srcs + (size_t)e * P.max_src;
    float *rho = (out_rho ? out_rho : rho_ev) + (size_t)e * nx * ny;
    float *ta = out_ta ? out_ta + (size_t)e * nx * ny : nullptr;
    float *tb = out_tb ? out_tb + (size_t)e * nx * ny : nullptr;
    int *corr = corr_scratch + (size_t)blockIdx.x * np * nx * ny;   // [plane][i][j], this CTA's
    const bool full = out_rho || ta || tb;
    const float kband = kln_event_band(P, rec);
    if (tid == 0) {
      s_status = rec.status;
      s_npend = 0;
    }
    KSum cm0, cm1, cm2, pre;   // pre: the density before NBD fluctuations (the zero-dN/dy test)
    const bool any = rec.imax > rec.imin && rec.jmax > rec.jmin;
    const int ti0 = rec.imin, tj0 = rec.jmin;
    const int nmt = any ? (rec.imax - rec.imin + kTM - 1) / kTM : 0;
    const int nnt = any ? (rec.jmax - rec.jmin + kTN - 1) / kTN : 0;
    // the splat sources (the leading nsplat records) are taken in windows of
    // kCap entries of the source array; one window (loaded once per event)
    // for all but the largest events
    const int nwin = (rec.nsplat + kCap - 1) / kCap;
    __syncthreads();
    // output grids: cells outside the tiles are zero (the tiles cover every window)
    if (full) {
      const int ci1 = any ? min(nx, ti0 + nmt * kTM) : 0, cj1 = any ? min(ny, tj0 + nnt * kTN) : 0;
      for (int i = wid; i < nx; i += kTW) {
        const bool rin = any && i >= ti0 && i < ci1;
        for (int j = lane; j < ny; j += 32) {
          if (rin && j >= tj0 && j < cj1) continue;
          rho[(size_t)i * ny + j] = 0.f;
          if (ta) ta[(size_t)i * ny + j] = 0.f;
          if (tb) tb[(size_t)i * ny + j] = 0.f;
        }
      }
    }
    // the splat sources of source-array window w, into the cache
    auto load_window = [&](int w) {
      int count = 0;
      const int lo = w * kCap, hi = min(rec.nsplat, lo + kCap);
      for (int b = lo; b < hi; b += kTT) {
        const int k = b + tid;
        const bool hit = k < hi && splat_source(S[k]);
        compact_append(hit, k - lo, list, s_wcnt, count);
      }
      for (int t = tid; t < count; t += kTT) {
        const Source &s = S[lo + list[t]];
        cache[t] = CSrc{(float)s.x, (float)s.y, s.weight, s.gi0, s.gfx, s.gj0, s.gfy, s.xl, s.xr, s.yl, s.yr,
                        s.kind, s.plane, lo + list[t]};
      }
      if (tid == 0) s_ncache = count;
      __syncthreads();
    };
    // ---- window cells beyond the cut, all (source, row) pairs of the event:
    // the corrections of the bounding box start at zero, then each pair (one
    // thread) finds the exact included interval of its window row and adds
    // the cells outside it
    for (int p = 0; p < np; p++)
      for (int i = rec.imin + wid; i < rec.imax; i += kTW)
        for (int j = rec.jmin + lane; j < rec.jmax; j += 32) corr[((size_t)p * nx + i) * ny + j] = 0;
    __syncthreads();
    for (int w = 0; w < nwin; w++) {
      load_window(w);
      const int nc = s_ncache, npair = nc * hmax;
      for (int q = tid; q < npair; q += kTT) {
        const int t = q / hmax;
        const CSrc &cs = cache[t];
        const int i = cs.xl + (q - t * hmax);
        if (i >= cs.xr) continue;
        const float dx = xg[i] - cs.xf;
        int ja, jb;
        cut_interval(P, &S[cs.idx].x, cs.kind, cs.yf, i, dx * dx, lim_lo, lim_hi, yg, inv_dy, ymin_f, cs.yl,
                     cs.yr, ja, jb);
        if (ja <= cs.yl && jb >= cs.yr) continue;
        const float exw = cs.w * gauss_grid((float)i, cs.gi0, cs.gfx, cx) * inv_corr_unit;
        int *crow = corr + ((size_t)cs.plane * nx + i) * ny;
        for (int j = cs.yl; j < ja; j++)
          atomicAdd(&crow[j], __float2int_rn(exw * gauss_grid((float)j, cs.gj0, cs.gfy, cy)));
        for (int j = jb; j < cs.yr; j++)
          atomicAdd(&crow[j], __float2int_rn(exw * gauss_grid((float)j, cs.gj0, cs.gfy, cy)));
      }
      __syncthreads();
    }

    for (int mt = 0; mt < nmt; mt++) {
      for (int nt = 0; nt < nnt; nt++) {
        const int i0 = ti0 + mt * kTM, j0 = tj0 + nt * kTN;
        const int i_own = i0 + r_own, c_lo = j0 + kQ * hc, c_hi = min(c_lo + kQ, ny);
        const int r_end = min(i0 + kTM, nx);
        for (int p = 0; p < np; p++) {
          float *own = stage + ((size_t)p * kTM + r_own) * kSP + kQ * hc;
#pragma unroll
          for (int c = 0; c < kQ; c++) own[c] = 0.f;
        }
        uint32_t used = 0;   // planes that received an MMA (block-uniform)
        for (int w = 0; w < nwin; w++) {
          if (nwin > 1) load_window(w);
          const int nc = s_ncache;
          // ---- tile list: cached sources reaching the tile, plane by plane
          // (plane 0 first), each plane in cache order
          int cnt_p[kMaxPlanes] = {0, 0};
          {
            for (int b = 0; b < nc; b += kTT) {
              const int t = b + tid;
              int pl = -1;
              if (t < nc) {
                const CSrc &cs = cache[t];
                if (cs.xl < i0 + kTM && cs.xr > i0 && cs.yl < j0 + kTN && cs.yr > j0) pl = cs.plane;
              }
              const unsigned b0 = __ballot_sync(0xffffffffu, pl == 0), b1 = __ballot_sync(0xffffffffu, pl == 1);
              if (lane == 0) s_wcnt[wid] = __popc(b0) | (__popc(b1) << 16);
              __syncthreads();
              int off0 = 0, off1 = 0, tot0 = 0, tot1 = 0;
#pragma unroll
              for (int q = 0; q < kTW; q++) {
                const int c = s_wcnt[q];
                off0 += q < wid ? (c & 0xffff) : 0;
                off1 += q < wid ? (c >> 16) : 0;
                tot0 += c & 0xffff;
                tot1 += c >> 16;
              }
              // plane 0 entries fill list[0 ..), plane 1 entries list[kCap - 1] downward
              const unsigned below = (1u << lane) - 1u;
              if (pl == 0) list[cnt_p[0] + off0 + __popc(b0 & below)] = (int16_t)t;
              if (pl == 1) list[kCap - 1 - (cnt_p[1] + off1 + __popc(b1 & below))] = (int16_t)t;
              __syncthreads();
              cnt_p[0] += tot0;
              cnt_p[1] += tot1;
            }
          }
          for (int p = 0; p < np; p++)
            if (cnt_p[p]) used |= 1u << p;
          // ---- 1. contraction on the tensor cores: the chunks of plane 0,
          // then of plane 1; chunk c is built into operand buffer c % 2
          // while the MMAs of chunk c-1 run, and chunk c-1 is then added
          // into its plane by the owner threads
          const int nch0 = (cnt_p[0] + kKC - 1) / kKC, nch = nch0 + (cnt_p[1] + kKC - 1) / kKC;
          auto src_of = [&](int p, int k) -> const CSrc & {   // k-th source of plane p's list
            return cache[p == 0 ? list[k] : list[kCap - 1 - k]];
          };
          int prev_plane = 0;
          for (int c = 0; c <= nch; c++) {
            if (c < nch) {
              const int b = c & 1;
              const int p = c < nch0 ? 0 : 1;
              const int c0 = (c < nch0 ? c : c - nch0) * kKC;
              const int kc = min(kKC, cnt_p[p] - c0), kpad = (kc + 7) & ~7;
              float *Ah = reinterpret_cast<float *>(smem + b * kOpSet);
              float *Al = Ah + kTM * kKC, *Bh = Al + kTM * kKC, *Bl = Bh + kTN * kKC;
              // A = rows x sources: w exp(-dx^2/2w^2) inside the row window
              for (int idx = tid; idx < kTM * kpad; idx += kTT) {
                const int core = idx >> 5, in = idx & 31;
                const int r = ((core & (kTM / 8 - 1)) << 3) + (in >> 2);
                const int q = ((core / (kTM / 8)) << 2) + (in & 3);
                const int i = i0 + r;
                float v = 0.f;
                if (q < kc) {
                  const CSrc &cs = src_of(p, c0 + q);
                  if (i >= cs.xl && i < cs.xr) v = cs.w * gauss_grid((float)i, cs.gi0, cs.gfx, cx);
                }
                const float h = tc::to_tf32(v);
                Ah[idx] = h;
                Al[idx] = tc::to_tf32(v - h);
              }
              // B = columns x sources: exp(-dy^2/2w^2) inside the column window
              for (int idx = tid; idx < kTN * kpad; idx += kTT) {
                const int core = idx >> 5, in = idx & 31;
                const int r = ((core & (kTN / 8 - 1)) << 3) + (in >> 2);
                const int q = ((core / (kTN / 8)) << 2) + (in & 3);
                const int j = j0 + r;
                float v = 0.f;
                if (q < kc) {
                  const CSrc &cs = src_of(p, c0 + q);
                  if (j >= cs.yl && j < cs.yr) v = gauss_grid((float)j, cs.gj0, cs.gfy, cy);
                }
                const float h = tc::to_tf32(v);
                Bh[idx] = h;
                Bl[idx] = tc::to_tf32(v - h);
              }
              tc::fence_proxy_async();
              tc::fence_before_sync();   // flush reads of this TMEM set (chunk c-2) are done
              __syncthreads();
              if (tid == 0 && !s_dead) {
                tc::fence_after_sync();
                const uint32_t sA = tc::smem_u32(Ah), sAl = sA + kOpA, sB = sA + 2 * kOpA, sBl = sB + kOpB;
                const uint32_t dm = tmem + (uint32_t)(2 * b * kTN);   // hi*hi
                const uint32_t dc = dm + (uint32_t)kTN;              // hi*lo + lo*hi
                for (int kk = 0; kk < kpad / 8; kk++) {
                  const uint64_t ah = tc::sdesc(sA + kk * 2 * kLboA, kLboA, kSbo);
                  const uint64_t al = tc::sdesc(sAl + kk * 2 * kLboA, kLboA, kSbo);
                  const uint64_t bh = tc::sdesc(sB + kk * 2 * kLboB, kLboB, kSbo);
                  const uint64_t bl = tc::sdesc(sBl + kk * 2 * kLboB, kLboB, kSbo);
                  tc::mma_tf32(dm, ah, bh, idesc, kk > 0);
                  tc::mma_tf32(dc, ah, bl, idesc, kk > 0);
                  tc::mma_tf32(dc, al, bh, idesc, 1);
                }
                tc::mma_commit(&s_bar[b]);
              }
            }
            if (c >= 1) {
              // chunk c-1 done (its operand buffer is free again): add its sums
              const int b = (c - 1) & 1;
              if (!tc::mbar_wait(&s_bar[b], phase[b], kMaxPolls)) {
                s_dead = 1;
                s_status = kErrMmaTimeout;
              }
              phase[b] ^= 1u;
              tc::fence_after_sync();
              if (!s_dead) {
                float v[kQ], x[kQ];
                tc::tmem_ld16(tmem + tm_lanes + (uint32_t)(2 * b * kTN + kQ * hc), v);
                tc::tmem_ld16(tmem + tm_lanes + (uint32_t)((2 * b + 1) * kTN + kQ * hc), x);
                float *own = stage + ((size_t)prev_plane * kTM + r_own) * kSP + kQ * hc;
#pragma unroll
                for (int k = 0; k < kQ; k++) own[k] += v[k] + x[k];
              }
            }
            prev_plane = c < nch0 ? 0 : 1;
          }
          __syncthreads();
        }
        // ---- 3. corner corrections into the planes (coalesced reads of the
        // L2-resident correction grid: the atomics came from other threads)
        __syncthreads();
        for (int p = 0; p < np; p++) {
          if (!((used >> p) & 1u)) continue;
          for (int r = wid; r < kTM; r += kTW) {
            const int i = i0 + r;
            if (i >= rec.imax) break;
            for (int c = lane; c < kTN; c += 32) {
              const int j = j0 + c;
              if (j < rec.jmax) stage[((size_t)p * kTM + r) * kSP + c] -= (float)__ldcg(corr + ((size_t)p * nx + i) * ny + j) * corr_unit;
            }
          }
        }
        __syncthreads();
        // ---- 4. post-op of the owned cells, outputs and centre-of-mass sums
        // (a warp owns 32 rows of the same columns: the loop is warp-uniform,
        // as the MC-KLN fix-up needs)
        {
          const float *sr = stage + (size_t)r_own * kSP + kQ * hc;
          for (int k = 0; k < kQ; k++) {
            const int j = c_lo + k;
            if (j >= c_hi) break;
            const bool inwin = i_own < rec.imax && j < rec.jmax;   // rec.imax <= nx
            float v = 0.f, t1 = 0.f, t2 = 0.f;
            int code = CELL_OK;
            if (inwin) {
              const float a0 = (used & 1u) ? fmaxf(sr[k], 0.f) : 0.f;
              const float a1 = np > 1 && (used & 2u) ? fmaxf(sr[kTM * kSP + k], 0.f) : 0.f;
              code = post_cell(P, np, a0, a1, 0.f, kband, v, t1, t2);
            }
            bool listed = false;
            if ((code & CELL_UNDECIDED) && kln_defer(s_pend, &s_npend, kPendCapTc, i_own, j, code, t1, t2)) {
              listed = true;
              code = CELL_OK;
            }
            if (P.which_mc_model == 1) kln_resolve_warp(P, rec, S, i_own, j, code, v, t1, t2);
            if (code == CELL_TABLE) s_status = 4;
            if (i_own >= nx || listed) continue;
            const size_t g = (size_t)i_own * ny + j;
            if (!inwin) {   // beyond every window: zero
              if (full) {
                rho[g] = 0.f;
                if (ta) ta[g] = 0.f;
                if (tb) tb[g] = 0.f;
              }
              continue;
            }
            if (P.nbd) {
              pre.add(v);
              v = nbd_cell(P, rec.ev, (uint32_t)g, v, t1, t2);
            }
            rho[g] = v;
            if (ta) ta[g] = t1;
            if (tb) tb[g] = t2;
            if (v != 0.f) {
              cm0.add(v);
              cm1.add(xg[i_own] * v);
              cm2.add(yg[j] * v);
            }
          }
        }
        __syncthreads();   // the cache window and the list are reused by the next tile
      }
    }
    // ---- the listed MC-KLN cells (s_npend is final after the tiles' last barrier)
    if (P.which_mc_model == 1) {
      const int npend = min(s_npend, kPendCapTc);
      if (npend > 0) {
        kln_finish_listed<kTW>(P, rec, S, s_pend, npend, rho, ta, tb, &s_status);
        __syncthreads();
        if (tid == 0) {
          const CmSums cs = kln_add_listed(s_pend, npend, ny, xg, yg, CmSums{cm0, cm1, cm2, pre});
          cm0 = cs.c0; cm1 = cs.c1; cm2 = cs.c2; pre = cs.pre;
        }
      }
    }
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
          for (int w = 0; w < kTW; w++) t += (double)red[w * 64 + lane].x + (double)red[w * 64 + lane].y;
        const double sa = __shfl_sync(0xffffffffu, t, 0), sd = __shfl_sync(0xffffffffu, t, 3);
        if (lane == 0) {
          s_cm[0] = sa;
          // MCnucl.cpp:812-816, on the density before the NBD fluctuations (:819)
          if (!((P.nbd ? sd : sa) * P.dx * P.dy >= 1e-15) && s_status == 0) s_status = 5;
        } else if (lane < 3) {
          s_cm[lane] = t / sa;
        }
      }
      __syncthreads();
    }
    if (tid == 0) {
      cm_ev[3 * (size_t)e] = s_cm[0];
      cm_ev[3 * (size_t)e + 1] = s_cm[1];
      cm_ev[3 * (size_t)e + 2] = s_cm[2];
    }
    if (tid == 0 && status) status[e] = s_status;
    __syncthreads();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (wid == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

constexpr int kCT = 256;   // threads of k_moments

// shared memory of k_moments: the hot-spot mask [nx][ceil(ny/32)] words, x - x_cm
// [nx], y - y_cm [ny rounded up to 32], then the reduction slots, 16-byte aligned
__host__ __device__ inline size_t moments_red_offset(int nx, int ny) {
  const size_t nyp = (ny + 31) / 32 * 32;
  const size_t b = sizeof(uint32_t) * (size_t)nx * (nyp / 32) + sizeof(float) * (nx + nyp);
  return (b + 15) / 16 * 16;
}

// ---------------------------------------------------------------- moments
// Eccentricities of each event from its density grid and centre-of-mass
// sums (MakeDensity::dumpEccentricities, src/MakeDensity.cpp:2244-2511).
template <int LO, int HI>
__global__ void __launch_bounds__(kCT) k_moments(DevParams P, int n_events, const EventRec *recs,
                                                 const Source *srcs, const float *rho_ev, const double *cm_ev,
                                                 double *out_ecc, EventQueue q) {
  extern __shared__ __align__(1024) unsigned char smem[];   // the same symbol as the splat's
  const int nx = P.nx, ny = P.ny;
  uint32_t *mask = reinterpret_cast<uint32_t *>(smem);
  float *xo = reinterpret_cast<float *>(smem + sizeof(uint32_t) * (size_t)nx * ((ny + 31) / 32));
  float *yo = xo + nx;
  float2 *red = reinterpret_cast<float2 *>(smem + moments_red_offset(nx, ny));
  const int tid = threadIdx.x;
  __shared__ int s_k;
  for (int k = queue_first(q, &s_k); k < n_events; k = queue_next(q, k, &s_k)) {
    const int e = queue_event(q, k);
    const EventRec rec = recs[e];
    const double tot0 = cm_ev[3 * (size_t)e], xc = cm_ev[3 * (size_t)e + 1], yc = cm_ev[3 * (size_t)e + 2];
    for (int i = tid; i < nx; i += kCT) xo[i] = (float)((P.xmin + i * P.dx) - xc);
    for (int j = tid; j < ny; j += kCT) yo[j] = (float)((P.ymin + j * P.dy) - yc);
    __syncthreads();
    moments<LO, HI, kCT>(P, rec, srcs + (size_t)e * P.max_src, rho_ev + (size_t)e * nx * ny, mask, xo, yo, red,
                         tot0, out_ecc + (size_t)e * kEccLen);
  }
}

size_t moments_smem(const DevParams &P) { return moments_red_offset(P.nx, P.ny) + sizeof(float2) * (kCT / 32) * 64; }

size_t grid_tc_smem(const DevParams &P) { return tc_layout(P.nx, P.ny, P.n_planes).total; }

bool grid_tc_supported(const DevParams &P) {
  // Gaussian profiles only (a disk profile is not a separable product), at
  // most two planes, source indices that fit the 16-bit lists, window
  // heights within a tile
  return P.shape_of_nucleons != 1 && P.shape_of_entropy != 1 && P.n_planes >= 1 &&
         P.n_planes <= kMaxPlanes && P.max_src <= 32767 && P.splat_mw <= kTM;
}


template <typename K>
static int blocks_per_sm(K kern, int threads, size_t smem) {
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
  int nb = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem) != cudaSuccess || nb < 1) nb = 1;
  return nb;
}

cudaError_t launch_grid_tc(const DevParams &P, int n_events, const EventRec *recs, const Source *srcs,
                           float *out_rho, float *out_ta, float *out_tb, float *rho_ev, int *corr_scratch,
                           double *cm_ev, double *out_ecc, int *status, int sms, cudaStream_t st,
                           const int *order, int *tickets) {
  if (n_events <= 0) return cudaSuccess;
  if (tickets) {
    cudaError_t e = cudaMemsetAsync(tickets, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return e;
  }
  // contraction, post-op, centre of mass
  {
    const size_t smem = grid_tc_smem(P);
    cudaError_t e = cudaFuncSetAttribute(k_grid_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_grid_tc<<<std::max(1, std::min(n_events, sms)), kTT, smem, st>>>(
        P, n_events, recs, srcs, out_rho, out_ta, out_tb, rho_ev, corr_scratch, cm_ev, status,
        EventQueue{order, tickets});
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (P.no_moments) return cudaSuccess;
  const size_t smem = moments_smem(P);
  const bool narrow = P.ecc_from >= 2 && P.ecc_to <= 5;
  auto kern = narrow ? k_moments<2, 5> : k_moments<1, 9>;
  const int nb = blocks_per_sm(kern, kCT, smem);
  kern<<<std::max(1, std::min(n_events, sms * nb)), kCT, smem, st>>>(
      P, n_events, recs, srcs, out_rho ? out_rho : rho_ev, cm_ev, out_ecc,
      EventQueue{order, tickets ? tickets + 1 : nullptr});
  return cudaGetLastError();
}

}  // namespace smc
