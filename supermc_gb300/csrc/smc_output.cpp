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
//
// The same tables in binary: NumPy .npy files (format version 1.0: magic,
// header dictionary, little-endian C-order data), one array per text file
// with the text file's columns and full precision.
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/supermc.h"

namespace {

// .npy header: 128 bytes in all (magic 6, version 2, length 2, dictionary
// padded with spaces, newline), so an append rewrites it in place
constexpr int kNpyHeader = 128;

std::string npy_dict(int elem_bytes, int ndim, const int64_t *shape, int64_t rows) {
  std::string d = std::string("{'descr': '<f") + (elem_bytes == 4 ? "4" : "8") + "', 'fortran_order': False, 'shape': (";
  for (int k = 0; k < ndim; k++) {
    d += std::to_string(k == 0 ? rows : shape[k]);
    d += (ndim == 1 || k + 1 < ndim) ? ", " : "";
  }
  return d + "), }";
}

bool npy_header(FILE *f, int elem_bytes, int ndim, const int64_t *shape, int64_t rows) {
  std::string d = npy_dict(elem_bytes, ndim, shape, rows);
  const size_t room = kNpyHeader - 10;
  if (d.size() + 1 > room) return false;
  d.append(room - 1 - d.size(), ' ');
  d += '\n';
  unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, (unsigned char)(room & 0xff),
                           (unsigned char)(room >> 8)};
  return std::fwrite(pre, 1, 10, f) == 10 && std::fwrite(d.data(), 1, d.size(), f) == d.size();
}

bool little_endian() {
  const uint16_t v = 1;
  unsigned char b;
  std::memcpy(&b, &v, 1);
  return b == 1;
}

// data in the file's little-endian byte order
bool npy_data(FILE *f, const void *data, int elem_bytes, size_t count) {
  if (little_endian()) return std::fwrite(data, (size_t)elem_bytes, count, f) == count;
  const unsigned char *p = static_cast<const unsigned char *>(data);
  std::vector<unsigned char> e((size_t)elem_bytes);
  for (size_t k = 0; k < count; k++) {
    for (int b = 0; b < elem_bytes; b++) e[b] = p[k * elem_bytes + elem_bytes - 1 - b];
    if (std::fwrite(e.data(), 1, e.size(), f) != e.size()) return false;
  }
  return true;
}

// rows already in an appendable file written by npy_write (its header must
// be this writer's, with the same type and trailing dimensions); -1: not one
int64_t npy_rows(FILE *f, int elem_bytes, int ndim, const int64_t *shape) {
  char h[kNpyHeader + 1] = {0};
  if (std::fread(h, 1, kNpyHeader, f) != (size_t)kNpyHeader) return -1;
  if ((unsigned char)h[0] != 0x93 || std::memcmp(h + 1, "NUMPY", 5) != 0 || h[6] != 1 || h[7] != 0) return -1;
  if ((unsigned char)h[8] + 256 * (unsigned char)h[9] != kNpyHeader - 10) return -1;
  const char *sh = std::strstr(h + 10, "'shape': (");
  if (!sh) return -1;
  long long rows = -1;
  if (std::sscanf(sh + 10, "%lld", &rows) != 1 || rows < 0) return -1;
  // the header this writer would write for that row count
  std::string want = npy_dict(elem_bytes, ndim, shape, rows);
  if (std::strncmp(h + 10, want.c_str(), want.size()) != 0) return -1;
  return rows;
}

smc_status npy_write(const char *filename, const void *data, int elem_bytes, int ndim, const int64_t *shape,
                     bool append) {
  if (!filename || (elem_bytes != 4 && elem_bytes != 8) || ndim < 1 || ndim > 4 || !shape) return SMC_ERR_ARGUMENT;
  size_t count = 1;
  for (int k = 0; k < ndim; k++) {
    if (shape[k] < 0) return SMC_ERR_ARGUMENT;
    count *= (size_t)shape[k];
  }
  if (count > 0 && !data) return SMC_ERR_ARGUMENT;
  FILE *f = append ? std::fopen(filename, "r+b") : nullptr;
  int64_t rows = 0;
  if (f) {
    rows = npy_rows(f, elem_bytes, ndim, shape);
    if (rows < 0) { std::fclose(f); return SMC_ERR_ARGUMENT; }
  } else {
    f = std::fopen(filename, "w+b");
    if (!f) return SMC_ERR_ARGUMENT;
    if (!npy_header(f, elem_bytes, ndim, shape, 0)) { std::fclose(f); return SMC_ERR_ARGUMENT; }
  }
  bool ok = std::fseek(f, 0, SEEK_END) == 0 && npy_data(f, data, elem_bytes, count);
  ok = ok && std::fseek(f, 0, SEEK_SET) == 0 && npy_header(f, elem_bytes, ndim, shape, rows + shape[0]);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? SMC_OK : SMC_ERR_ARGUMENT;
}

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

// the columns of one line of the per-order file (order 1..9) or of the
// all-orders line (order 10), as ecc_line prints them
int ecc_columns(const double *e, int order, const double *ori, double *out) {
  int c = 0;
  if (order < 10)
    for (int k = 0; k < 5; k++) out[c++] = e[5 * (order - 1) + k];
  else
    for (int k = 0; k < 45; k++) out[c++] = e[k];
  for (int k = 45; k < 49; k++) out[c++] = e[k];
  if (ori)
    for (int k = 0; k < 4; k++) out[c++] = ori[k];
  return c;
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

smc_status smc_write_npy(const char *filename, const void *data, int elem_bytes, int ndim, const int64_t *shape,
                         int append) {
  return npy_write(filename, data, elem_bytes, ndim, shape, append != 0);
}

smc_status smc_write_ecc_npy(const double *ecc, const double *orientation, int n, int from_order, int to_order,
                             const char *pattern) {
  if (!pattern || n < 0 || (n > 0 && !ecc) || from_order < 1 || to_order > 9 || from_order > to_order)
    return SMC_ERR_ARGUMENT;
  char path[4096];
  std::vector<double> rows;
  for (int order = from_order; order <= to_order + 1; order++) {
    const int which = order <= to_order ? order : 10;
    if (std::snprintf(path, sizeof(path), pattern, which) >= (int)sizeof(path)) return SMC_ERR_ARGUMENT;
    const int cols = (which < 10 ? 5 : 45) + 4 + (orientation ? 4 : 0);
    rows.assign((size_t)n * cols, 0.0);
    for (int e = 0; e < n; e++)
      ecc_columns(ecc + (size_t)e * kEccLen, which, orientation ? orientation + 4 * (size_t)e : nullptr,
                  rows.data() + (size_t)e * cols);
    const int64_t shape[2] = {n, cols};
    smc_status s = npy_write(path, rows.data(), 8, 2, shape, true);
    if (s) return s;
  }
  return SMC_OK;
}

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

smc_status smc_write_participant_table(const double *xy, const uint8_t *wounded, int A, int B, const char *filename) {
  if (!xy || !wounded || !filename || A < 0 || B < 0) return SMC_ERR_ARGUMENT;
  FILE *f = std::fopen(filename, "a");
  if (!f) return SMC_ERR_ARGUMENT;
  for (int k = 0; k < A + B; k++)
    if (wounded[k]) std::fprintf(f, "%10.3g   %10.3g   %d\n", xy[2 * k], xy[2 * k + 1], k < A ? 1 : 2);
  std::fclose(f);
  return SMC_OK;
}

smc_status smc_write_spectator_table(const double *xy, const uint8_t *wounded, int A, int B, double ecm,
                                     const char *filename) {
  if (!xy || !wounded || !filename || A < 0 || B < 0) return SMC_ERR_ARGUMENT;
  FILE *f = std::fopen(filename, "w");
  if (!f) return SMC_ERR_ARGUMENT;
  // the spectators' rapidity, +Y for the projectile, -Y for the target
  const double vz = std::sqrt(1. - 1. / ((ecm / 2.) * (ecm / 2.)));
  const double Y = 0.5 * std::log((1. + vz) / (1. - vz + 1e-100));
  for (int k = 0; k < A + B; k++)
    if (!wounded[k]) std::fprintf(f, "%10.4e  %.4e  %.4e\n", xy[2 * k], xy[2 * k + 1], k < A ? Y : -Y);
  std::fclose(f);
  return SMC_OK;
}

smc_status smc_write_density_pt(const float *data, int nx, int ny, int nbins, double npart, double scale,
                                const char *filename) {
  if (!data || !filename || nx < 1 || ny < 1 || nbins < 1) return SMC_ERR_ARGUMENT;
  FILE *f = std::fopen(filename, "w");
  if (!f) return SMC_ERR_ARGUMENT;
  std::fprintf(f, "%% <npart>= %g xmax= %d ymax= %d Ptmax= %d\n", npart, nx, ny, nbins);
  for (size_t c = 0; c < (size_t)nx * ny; c++) {
    for (int p = 0; p < nbins; p++) std::fprintf(f, "%22.12e", (double)data[c * nbins + p] * scale);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  return SMC_OK;
}

}  // extern "C"
