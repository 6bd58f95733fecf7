// Averaged-profile mode (MakeDensity::generate_profile_average,
// src/MakeDensity.cpp:736-2103; per-event loop :1240-1577).
//
// Per event and order n the reference recomputes the density, optionally
// recentres the sources on the density's centre of mass and re-splats
// (reaction-plane frame, :1291-1293), then rotates the sources to the
// order-n participant plane and re-splats (:1331-1333); the densities are
// averaged over all accepted events.  Here:
//   k_avg_init      per-source state: construction position and bounding box;
//   k_avg_transform centre of mass and angle of one event's grid
//                   (GlueDensity::calcCMAngle, src/GlueDensity.cpp:87-144) and
//                   the source transform of MCnucl::recenterGrid / rotateGrid
//                   (src/MCnucl.cpp:1119-1174) in FP64 with the reference's
//                   rounding, including Box2D's move arithmetic and the reset of
//                   a participant's box to its construction-time box
//                   (Particle::calculateBounds, src/Particle.cpp:94-99);
//   k_avg_accum     sum of the chunk's grids into FP64 accumulators.
// The splat itself is k_grid (without the eccentricity pass).
#include "smc_device.cuh"
#include "smc_kernels.h"

#include <algorithm>

namespace smc {

constexpr int kAT = 256;

__global__ void k_avg_init(DevParams P, int n_events, const EventRec *recs, const Source *srcs, AvgSrc *state) {
  const double c = 4 * fmax(P.width, P.quark_width);
  for (int e = blockIdx.x; e < n_events; e += gridDim.x) {
    const int ns = recs[e].nsrc;
    for (int k = threadIdx.x; k < ns; k += blockDim.x) {
      const Source &s = srcs[(size_t)e * P.max_src + k];
      AvgSrc a;
      if (s.kind & SRC_RAW_BASE) {
        // built at (bx, by): box = base U quark box there, then
        // Particle::setX / setY move it by Box2D::setCenter
        a.x0 = s.bx;
        a.y0 = s.by;
        const double xl = a.x0 - c, xr = a.x0 + c, yl = a.y0 - c, yr = a.y0 + c;
        const double xc = (xl + xr) / 2.0, yc = (yl + yr) / 2.0;
        a.bxl = xl + (s.x - xc); a.bxr = xr + (s.x - xc); a.bxc = s.x;
        a.byl = yl + (s.y - yc); a.byr = yr + (s.y - yc); a.byc = s.y;
      } else {
        a.x0 = s.x;
        a.y0 = s.y;
        a.bxl = s.x - c; a.bxr = s.x + c; a.byl = s.y - c; a.byr = s.y + c;   // Particle::Particle box
        a.bxc = (a.bxl + a.bxr) / 2.0;                                        // Box2D::overUnion centre
        a.byc = (a.byl + a.byr) / 2.0;
      }
      state[(size_t)e * P.max_src + k] = a;
    }
  }
}

struct DFs {
  float hi, lo;
};
__device__ __forceinline__ DFs dfs_add(DFs a, DFs b) {
  float s = a.hi + b.hi, bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
  float h = s + e;
  return {h, e - (h - s)};
}
__device__ double block_sum_df(float v, float c, float2 *red) {
  DFs x{v, -c};
  for (int o = 16; o; o >>= 1)
    x = dfs_add(x, DFs{__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)});
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = make_float2(x.hi, x.lo);
  __syncthreads();
  double s = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += (double)red[i].x + (double)red[i].y;
  return s;
}

struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c, t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// mode 0: recenter (MCnucl::recenterGrid); mode 1: rotate (MCnucl::rotateGrid);
// mode 2: only the frame.  With frame != NULL, frame[e] = (X, Y, cos, sin) of
// the centre of mass and the rotation the sources receive.
__global__ void __launch_bounds__(kAT) k_avg_transform(DevParams P, int n_events, EventRec *recs, Source *srcs,
                                                       AvgSrc *state, const float *rho, int order, int mode,
                                                       AvgFrame *frame) {
  __shared__ float2 red[kAT / 32];
  __shared__ double s_par[4];   // X, Y, cos, sin
  __shared__ int s_box[4];      // the event's new window bounds: imin, imax, jmin, jmax
  extern __shared__ float s_xy[];   // the cells' coordinates (float)(xmin + i dx), then y
  const int tid = threadIdx.x;
  const int nx = P.nx, ny = P.ny;
  const float inv_dx = (float)(1.0 / P.dx), inv_dy = (float)(1.0 / P.dy);
  const double d_max = P.shape_of_nucleons == 1 ? 2. * sqrt(P.dsq) : 5. * P.width;
  float *xg = s_xy, *yg = s_xy + nx;
  for (int i = tid; i < nx; i += kAT) xg[i] = (float)(P.xmin + i * P.dx);
  for (int j = tid; j < ny; j += kAT) yg[j] = (float)(P.ymin + j * P.dy);
  __syncthreads();
  // The density is zero outside the event's window box, and zero cells add
  // nothing: each thread visits the cells c = tid (mod kAT) of the full grid
  // in increasing order, as a walk over the whole grid would, but only those
  // inside the box (its first column of row i: jmin + ((tid - i ny - jmin)
  // mod kAT)), so the sums are those of the full walk.
  auto for_box = [&](const EventRec &r, auto &&f) {
    if (r.imax <= r.imin || r.jmax <= r.jmin) return;
    for (int i = r.imin; i < r.imax; i++) {
      const int row0 = i * ny + r.jmin;
      for (int j = r.jmin + ((tid - row0) & (kAT - 1)); j < r.jmax; j += kAT) f(i, j);
    }
  };
  static_assert((kAT & (kAT - 1)) == 0, "cells are dealt by a power-of-two stride");
  for (int e = blockIdx.x; e < n_events; e += gridDim.x) {
    const EventRec rec = recs[e];
    const float *g = rho + (size_t)e * nx * ny;
    // ---- centre of mass over the full grid (weights rho dx dy; dx dy cancels)
    Kahan sw, sx, sy;
    for_box(rec, [&](int i, int j) {
      const float v = g[(size_t)i * ny + j];
      if (v == 0.f) return;
      sw.add(v);
      sx.add(xg[i] * v);
      sy.add(yg[j] * v);
    });
    const double W = block_sum_df(sw.s, sw.c, red);
    const double SX = block_sum_df(sx.s, sx.c, red);
    const double SY = block_sum_df(sy.s, sy.c, red);
    if (!(W > 0)) {   // empty density: nothing to move (uniform over the block)
      if (frame && tid == 0) frame[e] = AvgFrame{0.0, 0.0, 1.0, 0.0};
      continue;
    }
    const double X = SX / W, Y = SY / W;
    // ---- order-n angle: sum r^n e^{in theta} rho about the centre (full grid)
    Kahan sr, si;
    const float Xf = (float)X, Yf = (float)Y;
    for_box(rec, [&](int i, int j) {
      const float v = g[(size_t)i * ny + j];
      if (v == 0.f) return;
      const float x = xg[i] - Xf, y = yg[j] - Yf;
      float zr = x, zi = y;
      for (int k = 1; k < order; k++) {
        const float t = zr * x - zi * y;
        zi = zr * y + zi * x;
        zr = t;
      }
      sr.add(zr * v);
      si.add(zi * v);
    });
    const double NR = block_sum_df(sr.s, sr.c, red);
    const double NI = block_sum_df(si.s, si.c, red);
    if (tid == 0) {
      const double ang = -atan2(-NI, -NR) / order;   // GlueDensity.cpp:140
      s_par[0] = X;
      s_par[1] = Y;
      s_par[2] = cos(ang);
      s_par[3] = sin(ang);
      s_box[0] = nx; s_box[1] = 0; s_box[2] = ny; s_box[3] = 0;
    }
    __syncthreads();
    const double cx = s_par[0], cy = s_par[1], cphi = s_par[2], sphi = s_par[3];
    if (frame && tid == 0) frame[e] = AvgFrame{cx, cy, cphi, sphi};
    if (mode == 2) continue;
    // ---- transform the sources (FP64, reference rounding)
    const double c4w = 4 * P.width, c4q = 4 * P.quark_width;
    for (int k = tid; k < rec.nsrc; k += kAT) {
      Source &s = srcs[(size_t)e * P.max_src + k];
      AvgSrc &a = state[(size_t)e * P.max_src + k];
      const int kind = s.kind & 15;
      // recenterGrid: setX(x - X) then setY(y - Y); boxes move by Box2D::setCenter
      double x = __dadd_rn(s.x, -cx);
      a.bxl = __dadd_rn(a.bxl, __dadd_rn(x, -a.bxc));
      a.bxr = __dadd_rn(a.bxr, __dadd_rn(x, -a.bxc));
      a.bxc = x;
      double y = __dadd_rn(s.y, -cy);
      a.byl = __dadd_rn(a.byl, __dadd_rn(y, -a.byc));
      a.byr = __dadd_rn(a.byr, __dadd_rn(y, -a.byc));
      a.byc = y;
      if (mode == 1) {
        // Point3D::rotate(cos(0), phi): x' = cphi x - sphi y, y' = sphi x + cphi y
        const double xr = __dadd_rn(__dmul_rn(cphi, x), -__dmul_rn(sphi, y));
        const double yr = __dadd_rn(__dmul_rn(sphi, x), __dmul_rn(cphi, y));
        x = xr;
        y = yr;
        // Particle::calculateBounds: construction box U quark box at the new position
        a.bxl = fmin(__dadd_rn(a.x0, -c4w), __dadd_rn(x, -c4q));
        a.bxr = fmax(__dadd_rn(a.x0, c4w), __dadd_rn(x, c4q));
        a.byl = fmin(__dadd_rn(a.y0, -c4w), __dadd_rn(y, -c4q));
        a.byr = fmax(__dadd_rn(a.y0, c4w), __dadd_rn(y, c4q));
        a.bxc = (a.bxl + a.bxr) / 2.0;
        a.byc = (a.byl + a.byr) / 2.0;
      }
      s.x = x;
      s.y = y;
      set_grid_offsets(s, P);
      // splat windows from the new geometry (src/MCnucl.cpp:829-832, :732-735, :450-453);
      // mask-only records keep their empty window
      if (kind == 3) continue;
      int xl, xr, yl, yr;
      if (kind == SRC_PART_BOX) {
        xl = trunc_index(a.bxl, P.xmin, P.dx, inv_dx); xr = trunc_index(a.bxr, P.xmin, P.dx, inv_dx);
        yl = trunc_index(a.byl, P.ymin, P.dy, inv_dy); yr = trunc_index(a.byr, P.ymin, P.dy, inv_dy);
        // After a rotation the box (construction box U quark box) can be far
        // wider than the splat's column table; only cells within the
        // inclusion radius of the source count (r <= 5w, or dc <= dsq for a
        // disk), so the window is cut to the rows / columns that can hold
        // one -- a superset, the per-cell test stays exact.
        const double R = (s.kind & 16) ? sqrt(P.dsq) : 5.0 * P.width;
        xl = max(xl, (int)floor((x - R - P.xmin) / P.dx - 0.01));
        xr = min(xr, (int)floor((x + R - P.xmin) / P.dx + 0.01) + 1);
        yl = max(yl, (int)floor((y - R - P.ymin) / P.dy - 0.01));
        yr = min(yr, (int)floor((y + R - P.ymin) / P.dy + 0.01) + 1);
      } else {
        xl = trunc_index(__dadd_rn(x, -d_max), P.xmin, P.dx, inv_dx);
        xr = trunc_index(__dadd_rn(x, d_max), P.xmin, P.dx, inv_dx);
        yl = trunc_index(__dadd_rn(y, -d_max), P.ymin, P.dy, inv_dy);
        yr = trunc_index(__dadd_rn(y, d_max), P.ymin, P.dy, inv_dy);
      }
      xl = max(0, xl); xr = min(nx, xr);
      yl = max(0, yl); yr = min(ny, yr);
      s.xl = (int16_t)xl; s.xr = (int16_t)xr;
      s.yl = (int16_t)yl; s.yr = (int16_t)yr;
      if (xr > xl && yr > yl) {
        atomicMin(&s_box[0], xl); atomicMax(&s_box[1], xr);
        atomicMin(&s_box[2], yl); atomicMax(&s_box[3], yr);
      }
    }
    __syncthreads();
    // the splat visits only the rows of the event's window bounds
    if (tid == 0) {
      recs[e].imin = s_box[0]; recs[e].imax = s_box[1];
      recs[e].jmin = s_box[2]; recs[e].jmax = s_box[3];
    }
  }
}

// Sources of a derived grid of the averaged mode, written to `out`:
//   mode 0, rho_binary (MCnucl::calculate_rho_binary, src/MCnucl.cpp:481-531):
//     the binary collisions with unit weight 1/(2 pi w^2) (10/sigma_in for
//     disk nucleons), plane 0;
//   mode 1, spectator densities (MCnucl::calculate_spectator_density,
//     src/MCnucl.cpp:534-614): the spectators, projectile into plane 1,
//     target into plane 2.
// Both cut at dc <= 25 w^2 (dc <= dsq for disks), the SRC_COLL rule; every
// other record becomes a mask-only record with an empty window.  The view's
// record carries the bounding box of its own windows.
__global__ void k_avg_view(DevParams P, int n_events, const EventRec *recs, const Source *in, Source *out, int mode,
                           EventRec *vrecs) {
  const bool disk = P.shape_of_nucleons == 1;
  const float w_unit = disk ? (float)(10.0 / P.sigin) : (float)P.peak;
  __shared__ int s_box[4];   // the view's window bounds: imin, imax, jmin, jmax
  for (int e = blockIdx.x; e < n_events; e += gridDim.x) {
    const int ns = recs[e].nsrc;
    if (threadIdx.x == 0) {
      s_box[0] = P.nx; s_box[1] = 0; s_box[2] = P.ny; s_box[3] = 0;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < ns; k += blockDim.x) {
      Source s = in[(size_t)e * P.max_src + k];
      const int kind = s.kind & 15;
      if (mode == 0 && (kind == SRC_COLL || kind == SRC_BINARY)) {
        s.kind = SRC_COLL | (disk ? 16 : 0);
        s.plane = 0;
        s.weight = w_unit;
      } else if (mode == 1 && kind == SRC_SPECT) {
        s.kind = SRC_COLL | (s.kind & 16);
        s.plane = 1 + s.plane;
      } else {
        s.kind = 3;
        s.xl = s.xr = s.yl = s.yr = 0;
      }
      if (s.kind != 3 && s.xr > s.xl && s.yr > s.yl) {
        atomicMin(&s_box[0], (int)s.xl); atomicMax(&s_box[1], (int)s.xr);
        atomicMin(&s_box[2], (int)s.yl); atomicMax(&s_box[3], (int)s.yr);
      }
      out[(size_t)e * P.max_src + k] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {   // the view's splat sources may lie anywhere in the records
      EventRec r = recs[e];
      r.nsplat = ns;
      r.imin = s_box[0]; r.imax = s_box[1]; r.jmin = s_box[2]; r.jmax = s_box[3];
      vrecs[e] = r;
    }
    __syncthreads();
  }
}

// acc[cell] += sum over the chunk's events of a_e[cell] * b_e[cell] (T_A T_B)
__global__ void k_avg_accum_prod(const float *a, const float *b, int n_events, size_t cells, double *acc) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (size_t)gridDim.x * blockDim.x) {
    Kahan k;
    for (int e = 0; e < n_events; e++) k.add(a[(size_t)e * cells + c] * b[(size_t)e * cells + c]);
    acc[c] += (double)k.s - (double)k.c;
  }
}

cudaError_t launch_avg_view(const DevParams &P, int n, const EventRec *recs, const Source *in, Source *out, int mode,
                            EventRec *vrecs, int grid, cudaStream_t st) {
  k_avg_view<<<grid, kAT, 0, st>>>(P, n, recs, in, out, mode, vrecs);
  return cudaGetLastError();
}

cudaError_t launch_avg_accum_prod(const float *a, const float *b, int n, size_t cells, double *acc, cudaStream_t st) {
  int blocks = (int)std::min<size_t>((cells + 255) / 256, 4096);
  k_avg_accum_prod<<<blocks, 256, 0, st>>>(a, b, n, cells, acc);
  return cudaGetLastError();
}

// acc[cell] += sum over the chunk's events of rho_e[cell] (Kahan in FP32 over
// the chunk, then one FP64 add per cell)
__global__ void k_avg_accum(const float *rho, int n_events, size_t cells, double *acc) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (size_t)gridDim.x * blockDim.x) {
    Kahan k;
    for (int e = 0; e < n_events; e++) k.add(rho[(size_t)e * cells + c]);
    acc[c] += (double)k.s - (double)k.c;
  }
}

// ---------------------------------------------------- centrality bins
// Events of the chunk in bin order (bin k: edges[k] <= Npart < edges[k+1]);
// seg[k] .. seg[k+1] delimit bin k in order[], events outside every bin are
// left out; within a bin the events keep their order (the bin sums are
// taken in that order).
__global__ void __launch_bounds__(1024) k_avg_bins(const EventRec *recs, int n, const int *edges, int nbins,
                                                   int *order, int *seg, int *counts) {
  // one CTA per bin b: the events of the bins before it give seg[b]; its own
  // events are then compacted in event order (bins are disjoint: the edges
  // do not decrease)
  __shared__ int s_w[32], s_v[32];
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int lo0 = edges[0], lob = edges[b], hib = edges[b + 1];
  auto npart = [&](int e, bool &in) {
    const EventRec &r = recs[e];
    in = r.ncoll > 0;
    return r.npart1 + r.npart2;
  };
  int before = 0, mine = 0;
  for (int e = tid; e < n; e += 1024) {
    bool in;
    const int np = npart(e, in);
    before += in && np >= lo0 && np < lob;
    mine += in && np >= lob && np < hib;
  }
  for (int o = 16; o; o >>= 1) {
    before += __shfl_xor_sync(0xffffffffu, before, o);
    mine += __shfl_xor_sync(0xffffffffu, mine, o);
  }
  if (lane == 0) { s_w[wid] = before; s_v[wid] = mine; }
  __syncthreads();
  int base = 0, total = 0;
  for (int q = 0; q < 32; q++) { base += s_w[q]; total += s_v[q]; }
  __syncthreads();
  if (tid == 0) {
    seg[b] = base;
    counts[b] += total;
    if (b == nbins - 1) seg[nbins] = base + total;
  }
  for (int e0 = 0; e0 < n; e0 += 1024) {
    const int e = e0 + tid;
    bool f = false;
    if (e < n) {
      bool in;
      const int np = npart(e, in);
      f = in && np >= lob && np < hib;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) s_w[wid] = __popc(bal);
    __syncthreads();
    int off = 0, tot = 0;
    for (int q = 0; q < 32; q++) {
      const int c = s_w[q];
      off += q < wid ? c : 0;
      tot += c;
    }
    if (f) order[base + off + __popc(bal & ((1u << lane) - 1u))] = e;
    base += tot;
    __syncthreads();
  }
}

// acc[b][cell] (FP32 sum, compensation) += the chunk's bin-b events at the
// cell: with frame, the value of the event's density at the cell's preimage
// under the recentring and rotation, R(-phi) (x', y') + (X, Y), by bilinear
// interpolation (corners beyond the grid read zero); without, the cell's
// value.  One thread per output cell, 16 x 16 cells per CTA, events in bin
// order with one compensated sum in registers.  The CTA stages the events
// 256 at a time: each thread tests one event against the tile (the
// preimage of the tile's corners against the event's window box, outside
// which its density is zero) and the events that can reach the tile are
// compacted in order into shared memory with their frames; the cells then
// read four events' values at a time and add them in order.
__device__ __forceinline__ float binned_value(const float *G, int nx, int ny, float4 f, float xo, float yo,
                                              float inv_dx, float inv_dy, bool resample, int i, int j) {
  if (!resample) return G[(size_t)i * ny + j];
  // preimage in grid units (f: cos, sin, X - xmin, Y - ymin)
  const float px = (f.x * xo + f.y * yo + f.z) * inv_dx;
  const float py = (-f.y * xo + f.x * yo + f.w) * inv_dy;
  const float fx = floorf(px), fy = floorf(py);
  const int i0 = (int)fx, j0 = (int)fy;
  const float tx = px - fx, ty = py - fy;
  if (!(i0 >= -1 && i0 < nx && j0 >= -1 && j0 < ny)) return 0.f;
  const bool xa = i0 >= 0, xb = i0 + 1 < nx, ya = j0 >= 0, yb = j0 + 1 < ny;
  const float v00 = xa && ya ? G[(size_t)i0 * ny + j0] : 0.f;
  const float v01 = xa && yb ? G[(size_t)i0 * ny + j0 + 1] : 0.f;
  const float v10 = xb && ya ? G[(size_t)(i0 + 1) * ny + j0] : 0.f;
  const float v11 = xb && yb ? G[(size_t)(i0 + 1) * ny + j0 + 1] : 0.f;
  return (1.f - tx) * ((1.f - ty) * v00 + ty * v01) + tx * ((1.f - ty) * v10 + ty * v11);
}

// The events of each bin are split into gridDim.z consecutive slices, one
// per CTA of the tile (the central tiles see nearly every event: one CTA
// walking all of them would be the whole kernel's critical path).  One
// slice: the sums go straight into acc; more: slice s writes its
// compensated sums to part[s][bin][cell] for k_avg_merge.
__global__ void __launch_bounds__(256) k_avg_binned(DevParams P, const EventRec *recs, const float *rho,
                                                   const AvgFrame *frame, const int *order, const int *seg,
                                                   int nbins, float2 *acc, float2 *part) {
  __shared__ float4 s_fr[256];
  __shared__ int s_ev[256];
  __shared__ int s_wc[8];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int i = blockIdx.y * 16 + (tid >> 4), j = blockIdx.x * 16 + (tid & 15);
  const int ti0 = blockIdx.y * 16, tj0 = blockIdx.x * 16;   // the tile's first cell
  const int nx = P.nx, ny = P.ny;
  const bool in = i < nx && j < ny;
  const size_t g = (size_t)nx * ny;
  const float xo = (float)(P.xmin + i * P.dx), yo = (float)(P.ymin + j * P.dy);
  const float inv_dx = (float)(1.0 / P.dx), inv_dy = (float)(1.0 / P.dy);
  const float xmin = (float)P.xmin, ymin = (float)P.ymin;
  const bool resample = frame != nullptr;
  const int slices = gridDim.z, sl = blockIdx.z;
  for (int b = 0; b < nbins; b++) {
    Kahan k;
    const int b0 = seg[b], n_b = seg[b + 1] - b0;
    const int e0 = b0 + (int)((long long)n_b * sl / slices), e1 = b0 + (int)((long long)n_b * (sl + 1) / slices);
    for (int q0 = e0; q0 < e1; q0 += 256) {
      // ---- stage: which of the next 256 events can reach this tile
      bool hit = false;
      float4 fr = make_float4(1.f, 0.f, 0.f, 0.f);
      int e = 0;
      if (q0 + tid < e1) {
        e = order[q0 + tid];
        const EventRec r = recs[e];
        if (resample) {
          const AvgFrame f = frame[e];
          fr = make_float4((float)f.c, (float)f.s, (float)f.x - xmin, (float)f.y - ymin);
          float lo_x = 1e30f, hi_x = -1e30f, lo_y = 1e30f, hi_y = -1e30f;
#pragma unroll
          for (int corner = 0; corner < 4; corner++) {
            const float cx = (float)(P.xmin + (ti0 + (corner & 1) * 15) * P.dx);
            const float cy = (float)(P.ymin + (tj0 + (corner >> 1) * 15) * P.dy);
            const float qx = (fr.x * cx + fr.y * cy + fr.z) * inv_dx;
            const float qy = (-fr.y * cx + fr.x * cy + fr.w) * inv_dy;
            lo_x = fminf(lo_x, qx); hi_x = fmaxf(hi_x, qx);
            lo_y = fminf(lo_y, qy); hi_y = fmaxf(hi_y, qy);
          }
          // bilinear corners floor(p), floor(p) + 1 against the box [imin, imax)
          hit = !(hi_x < r.imin - 1 || lo_x >= r.imax || hi_y < r.jmin - 1 || lo_y >= r.jmax);
        } else {
          hit = !(ti0 >= r.imax || ti0 + 16 <= r.imin || tj0 >= r.jmax || tj0 + 16 <= r.jmin);
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, hit);
      if (lane == 0) s_wc[wid] = __popc(bal);
      __syncthreads();
      int off = 0, tot = 0;
#pragma unroll
      for (int w = 0; w < 8; w++) {
        const int c = s_wc[w];
        off += w < wid ? c : 0;
        tot += c;
      }
      if (hit) {
        const int p = off + __popc(bal & ((1u << lane) - 1u));
        s_ev[p] = e;
        s_fr[p] = fr;
      }
      __syncthreads();
      // ---- accumulate in event order, four loads in flight
      if (in) {
        int m = 0;
        for (; m + 4 <= tot; m += 4) {
          float v[4];
#pragma unroll
          for (int u = 0; u < 4; u++)
            v[u] = binned_value(rho + (size_t)s_ev[m + u] * g, nx, ny, s_fr[m + u], xo, yo, inv_dx, inv_dy,
                                resample, i, j);
#pragma unroll
          for (int u = 0; u < 4; u++) k.add(v[u]);
        }
        for (; m < tot; m++)
          k.add(binned_value(rho + (size_t)s_ev[m] * g, nx, ny, s_fr[m], xo, yo, inv_dx, inv_dy, resample, i, j));
      }
      __syncthreads();   // the staged events are read before the next stage
    }
    if (in && slices > 1) {
      part[((size_t)sl * nbins + b) * g + (size_t)i * ny + j] = make_float2(k.s, k.c);
    } else if (in && e1 > e0) {
      // merge the chunk's compensated sum into the accumulator's
      float2 a = acc[(size_t)b * g + (size_t)i * ny + j];
      const float y = (k.s - k.c) - a.y, t = a.x + y;
      a.y = (t - a.x) - y;
      a.x = t;
      acc[(size_t)b * g + (size_t)i * ny + j] = a;
    }
  }
}

// acc[b][cell] += the slices' compensated sums, in slice order (empty
// slices, exactly zero, are passed over)
__global__ void k_avg_merge(const float2 *part, int slices, size_t cells_all, float2 *acc) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells_all; c += (size_t)gridDim.x * blockDim.x) {
    float2 a = acc[c];
    for (int s = 0; s < slices; s++) {
      const float2 p = part[(size_t)s * cells_all + c];
      if (p.x == 0.f && p.y == 0.f) continue;
      const float y = (p.x - p.y) - a.y, t = a.x + y;
      a.y = (t - a.x) - y;
      a.x = t;
    }
    acc[c] = a;
  }
}

int avg_binned_slices(const DevParams &P) {
  const int tiles = ((P.nx + 15) / 16) * ((P.ny + 15) / 16);
  return std::max(1, std::min(8, (4096 + tiles - 1) / tiles));
}

cudaError_t launch_avg_bins(const EventRec *recs, int n, const int *edges, int nbins, int *order, int *seg,
                            int *counts, cudaStream_t st) {
  k_avg_bins<<<nbins, 1024, 0, st>>>(recs, n, edges, nbins, order, seg, counts);
  return cudaGetLastError();
}

cudaError_t launch_avg_binned(const DevParams &P, const EventRec *recs, const float *rho, const AvgFrame *frame,
                              const int *order, const int *seg, int nbins, float2 *acc, float2 *part, cudaStream_t st) {
  const int slices = part ? avg_binned_slices(P) : 1;
  dim3 grid((P.ny + 15) / 16, (P.nx + 15) / 16, slices);
  k_avg_binned<<<grid, 256, 0, st>>>(P, recs, rho, frame, order, seg, nbins, acc, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || slices == 1) return e;
  const size_t all = (size_t)nbins * P.nx * P.ny;
  k_avg_merge<<<(int)std::min<size_t>((all + 255) / 256, 8192), 256, 0, st>>>(part, slices, all, acc);
  return cudaGetLastError();
}

cudaError_t launch_avg_init(const DevParams &P, int n, const EventRec *recs, const Source *srcs, AvgSrc *state,
                            int grid, cudaStream_t st) {
  k_avg_init<<<grid, kAT, 0, st>>>(P, n, recs, srcs, state);
  return cudaGetLastError();
}
cudaError_t launch_avg_transform(const DevParams &P, int n, EventRec *recs, Source *srcs, AvgSrc *state,
                                 const float *rho, int order, int mode, int grid, cudaStream_t st, AvgFrame *frame) {
  const size_t smem = sizeof(float) * (size_t)(P.nx + P.ny);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(k_avg_transform, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_avg_transform<<<grid, kAT, smem, st>>>(P, n, recs, srcs, state, rho, order, mode, frame);
  return cudaGetLastError();
}
cudaError_t launch_avg_accum(const float *rho, int n, size_t cells, double *acc, cudaStream_t st) {
  int blocks = (int)std::min<size_t>((cells + 255) / 256, 4096);
  k_avg_accum<<<blocks, 256, 0, st>>>(rho, n, cells, acc);
  return cudaGetLastError();
}

}  // namespace smc
