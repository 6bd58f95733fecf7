// The reference's MakeDensity call surface (src/MakeDensity.h:43-63) over the
// GPU library's C ABI (include/supermc.h): the operations main() runs
// (src/main.cpp:42-61) write the same files under data/.
//   generateEccTable          operation 9: data/sn_ecc_eccp_<order>.dat
//   generate_profile_ebe      operation 1: data/sd_event_<n>_block.dat / _4col.dat,
//                             data/binary.dat, wounded.data, nucl1.data, nucl2.data
//   generate_profile_ebe_Jet  operation 2: per event data/ParticipantTable_event_<n>.dat,
//                             Spectators_event_<n>.dat, BinaryCollisionTable_event_<n>.dat,
//                             sn_ecc_eccp_<order>_event_<n>.dat, sd_event_<n>_block/_4col,
//                             rho_binary_event_<n>_*, nuclear_thickness_TA/TB_event_<n>_*,
//                             rhob_event_<n>_*, spectator_density_A/B_event_<n>_*
//   generate_profile_average  operation 3: data/sdAvg[_RP]_order_<n>_block.dat / _4col.dat and
//                             the TATB, rho_binary, nuclear_thickness, spectator_density means
// With the key use_binary = 1 (no reference counterpart) each of these tables
// is written as a NumPy .npy file of the same name (.npy for .dat / .data)
// holding the text file's columns at full precision.
// Parameters are the reference's parameters.dat keys; a key the file does not
// set takes the value the reference ships in its parameters.dat.  Failures
// throw smc::Error (the reference exits).
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/supermc.h"
#include "ParameterReader.h"

namespace smc {

struct Error : std::runtime_error {
  smc_status status;
  Error(smc_status s, const std::string &what);
};

// smc_params from the reader (reference defaults for absent keys)
smc_params params_from(const ParameterReader &p);

// The configuration tables of the light nuclei among the projectile and the
// target (A = 3, 4, 12, 16), read from tables/ of the working directory as
// the Nucleus constructor reads them (src/Nucleus.cpp:150-164, 383-478); a
// missing or unreadable file throws (the reference exits).
void load_light_tables(void *ctx, const smc_params &p);

class MakeDensity {
 public:
  explicit MakeDensity(ParameterReader *reader);   // MakeDensity::MakeDensity, src/MakeDensity.cpp:21-134
  ~MakeDensity();
  MakeDensity(const MakeDensity &) = delete;
  MakeDensity &operator=(const MakeDensity &) = delete;

  void generateEccTable(int nevent);           // src/MakeDensity.cpp:2103-2200
  void generate_profile_ebe(int nevent);       // :501-694
  void generate_profile_ebe_Jet(int nevent);   // :148-498 (operation 2)
  void generate_profile_average(int nevent);   // :736-2103 (integrated-p_T entropy means)
  // The per-event helpers the operations use, on the library's results:
  // setSd (src/MakeDensity.cpp:2514-2522): sd = getRho * finalFactor
  void setSd(const float *rho, double *sd) const;
  // gettotaldSdy (:2557-2567): sum of getRho dx dy
  double gettotaldSdy(const float *rho) const;
  // dumpDensityBlock / dumpDensity4Col (:2597-2609, :2573-2595) of one [nx][ny] grid
  void dumpDensityBlock(const char *filename, const double *grid) const;
  void dumpDensity4Col(const char *filename, const double *grid, double npart = 0.0) const;
  // dumpEccentricities (:2244-2511): appends n events' lines to
  // <base_filename>_<order>.dat, from the ecc[49] rows the library computes
  // from each event's density (orientation [n][4]: the deformed layout)
  void dumpEccentricities(const char *base_filename, const double *ecc, int n, int from_order, int to_order,
                          const double *orientation = nullptr) const;

  // events per library call (host buffers are sized for one call)
  void setBatch(int events) { batch_ = events; }
  void *context() const { return ctx_; }
  const smc_info &info() const { return info_; }
  // a failed call's status as smc::Error
  static void check_status(smc_status s, const char *what);

 private:
  ParameterReader *reader_;
  void *ctx_ = nullptr;
  smc_info info_{};
  smc_params params_{};
  int batch_ = 16384;
  bool binary_ = false;   // use_binary = 1: .npy files in place of the text files
  void check(smc_status s, const char *what) const;
  void write_nucleon_npy(const double *xy, const uint8_t *wounded);
};

}  // namespace smc
