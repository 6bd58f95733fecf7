// Per-cell p_T-differential MC-KLN densities: MCnucl::setDensity(iy, ipt)
// for every p_T bin (src/MCnucl.cpp:626-687, the ipt >= 0 branch): the
// six-point interpolation (src/arsenal.cpp:33-54) of the p_T-differential
// table (k_kln_pt_table) in the table cell the cell's T_A, T_B select --
// the cell of the p_T-integrated lookup: floor(T/dT) from the FP32
// thickness where it is decided there, else from FP64 sums of the
// thickness records (post_cell, thickness_fp64).  The reference's
// per-cell fluctuations act on the p_T-integrated density only
// (MCnucl::fluctuateCurrentDensity, :869-905), so none apply here.
#include "grid_common.cuh"
#include "smc_kernels.h"

namespace smc {

constexpr int kPT = 256;

// one CTA per event at a time (static stride); warps take the rows of the
// event's window bounding box, lanes its columns.  ta, tb: the event's
// thickness outputs of the splat; out: [n][nx][ny][nbins], zeroed outside
// the bounding box by the launcher.
__global__ void __launch_bounds__(kPT) k_kln_pt_cells(DevParams P, int n, const EventRec *recs, const Source *srcs,
                                                      const float *ta, const float *tb, const float *table,
                                                      int nbins, float *out, int *status) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nx = P.nx, ny = P.ny, tm = P.kln_tmax;
  for (int e = blockIdx.x; e < n; e += gridDim.x) {
    const EventRec rec = recs[e];
    const Source *S = srcs + (size_t)e * P.max_src;
    const float band = kln_event_band(P, rec);
    const size_t g0 = (size_t)e * nx * ny;
    const int base0 = rec.nsplat - rec.npart1 - rec.npart2, base1 = base0 + rec.npart1;
    for (int i = rec.imin + wid; i < rec.imax; i += kPT / 32) {
      for (int jb = rec.jmin; jb < rec.jmax; jb += 32) {
        const int j = jb + lane;
        const bool ok = j < rec.jmax;
        float t1 = ok ? ta[g0 + (size_t)i * ny + j] : 0.f, t2 = ok ? tb[g0 + (size_t)i * ny + j] : 0.f;
        float v, o1, o2;
        int code = ok ? post_cell(P, 2, t1, t2, 0.f, band, v, o1, o2) : CELL_OK;
        // table cell and offsets, FP32 where post_cell decided them
        int ii = 0, jj = 0;
        float fi = 0.f, fj = 0.f;
        bool live = ok && code == CELL_OK && o1 > 0.f && o2 > 0.f;
        if (live) {
          const float di = o1 * P.kln_inv_dT_f, dj = o2 * P.kln_inv_dT_f;
          ii = (int)di;
          jj = (int)dj;
          fi = di - floorf(di);
          fj = dj - floorf(dj);
        }
        // the undecided cells, one at a time by the whole warp, from FP64 sums
        unsigned m = __ballot_sync(0xffffffffu, (code & CELL_UNDECIDED) != 0);
        while (m) {
          const int src = __ffs(m) - 1;
          m &= m - 1u;
          const int need = __shfl_sync(0xffffffffu, code, src);
          double da = (double)__shfl_sync(0xffffffffu, t1 < P.kln_tzero ? 0.f : t1, src);
          double db = (double)__shfl_sync(0xffffffffu, t2 < P.kln_tzero ? 0.f : t2, src);
          const int cj = jb + src;
          if (need & CELL_NEED_A) da = thickness_fp64(P, S, base0, rec.npart1, 0, i, cj);
          if (need & CELL_NEED_B) db = thickness_fp64(P, S, base1, rec.npart2, 1, i, cj);
          if (lane == src) {
            const double di = da / P.kln_dT, dj = db / P.kln_dT;
            code = (di >= tm - 2 || dj >= tm - 2) ? CELL_TABLE : CELL_OK;
            live = code == CELL_OK && da != 0.0 && db != 0.0;
            if (live) {
              ii = (int)floor(di);
              jj = (int)floor(dj);
              fi = (float)(di - ii);
              fj = (float)(dj - jj);
            }
          }
        }
        if (code == CELL_TABLE && status) atomicMax(status + e, 4);   // per-event code of a thickness beyond the table
        if (live) {
          float *o = out + (g0 + (size_t)i * ny + j) * nbins;
          const float *T = table + ((size_t)ii * tm + jj) * nbins;
          const size_t r1 = (size_t)tm * nbins;
          for (int p = 0; p < nbins; p++)
            o[p] = six_point(fi, fj, __ldg(T + p), __ldg(T + nbins + p), __ldg(T + 2 * nbins + p), __ldg(T + r1 + p),
                             __ldg(T + r1 + nbins + p), __ldg(T + 2 * r1 + p));
        }
      }
    }
  }
}

cudaError_t launch_kln_pt_cells(const DevParams &P, int n, const EventRec *recs, const Source *srcs, const float *ta,
                                const float *tb, const float *table, int nbins, float *out, int *status, int grid,
                                cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n * P.nx * P.ny * nbins, st);
  if (e != cudaSuccess) return e;
  k_kln_pt_cells<<<grid, kPT, 0, st>>>(P, n, recs, srcs, ta, tb, table, nbins, out, status);
  return cudaGetLastError();
}

}  // namespace smc
