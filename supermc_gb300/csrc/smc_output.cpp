// Text outputs in the layouts the reference writes, from the results of the
// C ABI calls (host code; no GPU needed).
//
//   sn_ecc_eccp_<order>.dat, sn_ecc_eccp_10.dat   MakeDensity::dumpEccentricities,
//                                                 src/MakeDensity.cpp:2432-2500
//   sd_event_<n>_block.dat                        MakeDensity::dumpDensityBlock,
//                                                 src/MakeDensity.cpp:2597-2609
//   sd_event_<n>_4col.dat                         MakeDensity::dumpDensity4Col,
//                                                 src/MakeDensity.cpp:2573-2595
//
// The reference formats with iostreams, setprecision(p) << setw(w) in the
// default float field, which is C's "%w.pg".
#include <cstdio>

#include "../../include/supermc.h"

namespace {

constexpr int kEccLen = 49;

// writes a line of the per-order file (order in 1..9) or, for order 10, the
// line with all orders; fields as in dumpEccentricities, plus the four
// orientation fields of the deformed layout when ori is given
void ecc_line(FILE *f, const double *e, int order, const double *ori) {
  if (order < 10) {
    const double *o = e + 5 * (order - 1);
    std::fprintf(f, "%16.8g%16.8g%16.8g%16.8g%16.8g", o[0], o[1], o[2], o[3], o[4]);
  } else {
    for (int k = 0; k < 45; k++) std::fprintf(f, "%16.8g", e[k]);
  }
  std::fprintf(f, "%10.5g%10.5g%16.8g%16.8g", e[45], e[46], e[47], e[48]);
  if (ori) std::fprintf(f, "%16.8g%16.8g%16.8g%16.8g", ori[0], ori[1], ori[2], ori[3]);
  std::fprintf(f, "\n");
}

smc_status write_ecc(const double *ecc, const double *ori, int n, int from_order, int to_order, const char *pattern) {
  if (!pattern || n < 0 || (n > 0 && !ecc) || from_order < 1 || to_order > 9 || from_order > to_order)
    return SMC_ERR_ARGUMENT;
  char path[4096];
  for (int order = from_order; order <= to_order + 1; order++) {
    const int which = order <= to_order ? order : 10;
    if (std::snprintf(path, sizeof(path), pattern, which) >= (int)sizeof(path)) return SMC_ERR_ARGUMENT;
    FILE *f = std::fopen(path, "a");
    if (!f) return SMC_ERR_ARGUMENT;
    for (int e = 0; e < n; e++) ecc_line(f, ecc + (size_t)e * kEccLen, which, ori ? ori + 4 * (size_t)e : nullptr);
    std::fclose(f);
  }
  return SMC_OK;
}

}  // namespace

extern "C" {

smc_status smc_write_ecc(const double *ecc, int n, int from_order, int to_order, const char *pattern) {
  return write_ecc(ecc, nullptr, n, from_order, to_order, pattern);
}

smc_status smc_write_ecc_deformed(const double *ecc, const double *orientation, int n, int from_order, int to_order,
                                  const char *pattern) {
  if (n > 0 && !orientation) return SMC_ERR_ARGUMENT;
  return write_ecc(ecc, orientation, n, from_order, to_order, pattern);
}

smc_status smc_write_density_block(const double *grid, int nx, int ny, const char *filename) {
  if (!grid || !filename || nx < 1 || ny < 1) return SMC_ERR_ARGUMENT;
  FILE *f = std::fopen(filename, "w");
  if (!f) return SMC_ERR_ARGUMENT;
  for (int i = 0; i < nx; i++) {
    for (int j = 0; j < ny; j++) std::fprintf(f, "%22.12g", grid[(size_t)i * ny + j]);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  return SMC_OK;
}

smc_status smc_write_density_4col(const double *grid, int nx, int ny, double xmin, double ymin, double dx, double dy,
                                  double rapidity, double npart, const char *filename) {
  if (!grid || !filename || nx < 1 || ny < 1) return SMC_ERR_ARGUMENT;
  FILE *f = std::fopen(filename, "w");
  if (!f) return SMC_ERR_ARGUMENT;
  std::fprintf(f, "# <npart>= %g xmax= %d ymax= %d\n", npart, nx, ny);
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      const double x = xmin + i * dx, y = ymin + j * dy;
      std::fprintf(f, "%10.3g%10.3g%10.3g%22.12g\n", rapidity, x, y, grid[(size_t)i * ny + j]);
    }
  std::fclose(f);
  return SMC_OK;
}

smc_status smc_write_binary_table(const double *xy, int ncoll, const char *filename) {
  if (!filename || ncoll < 0 || (ncoll > 0 && !xy)) return SMC_ERR_ARGUMENT;
  FILE *f = std::fopen(filename, "a");
  if (!f) return SMC_ERR_ARGUMENT;
  for (int c = 0; c < ncoll; c++) std::fprintf(f, "%10.3g%10.3g\n", xy[2 * c], xy[2 * c + 1]);
  std::fclose(f);
  return SMC_OK;
}

smc_status smc_write_nucleon_tables(const double *xy, const uint8_t *wounded, int A, int B, const char *participants,
                                    const char *proj, const char *targ) {
  if (!xy || A < 0 || B < 0 || (participants && !wounded)) return SMC_ERR_ARGUMENT;
  if (participants) {
    FILE *f = std::fopen(participants, "w");
    if (!f) return SMC_ERR_ARGUMENT;
    for (int k = 0; k < A + B; k++)
      if (wounded[k]) std::fprintf(f, "%10.3g   %10.3g   %d\n", xy[2 * k], xy[2 * k + 1], k < A ? 1 : 2);
    std::fclose(f);
  }
  const char *names[2] = {proj, targ};
  for (int w = 0; w < 2; w++) {
    if (!names[w]) continue;
    FILE *f = std::fopen(names[w], "w");
    if (!f) return SMC_ERR_ARGUMENT;
    const int k0 = w ? A : 0, k1 = w ? A + B : A;
    for (int k = k0; k < k1; k++) std::fprintf(f, "%10.3g%10.3g\n", xy[2 * k], xy[2 * k + 1]);
    std::fclose(f);
  }
  return SMC_OK;
}

}  // extern "C"
