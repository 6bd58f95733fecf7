// The reference's MakeDensity call surface (src/MakeDensity.h:43-63) over the
// GPU library's C ABI (include/supermc.h): the operations main() runs
// (src/main.cpp:42-61) write the same files under data/.
//   generateEccTable          operation 9: data/sn_ecc_eccp_<order>.dat
//   generate_profile_ebe      operation 1: data/sd_event_<n>_block.dat / _4col.dat,
//                             data/binary.dat, wounded.data, nucl1.data, nucl2.data
//   generate_profile_average  operation 3: data/sdAvg[_RP]_order_<n>_block.dat / _4col.dat and
//                             the TATB, rho_binary, nuclear_thickness, spectator_density means
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

class MakeDensity {
 public:
  explicit MakeDensity(ParameterReader *reader);   // MakeDensity::MakeDensity, src/MakeDensity.cpp:21-134
  ~MakeDensity();
  MakeDensity(const MakeDensity &) = delete;
  MakeDensity &operator=(const MakeDensity &) = delete;

  void generateEccTable(int nevent);           // src/MakeDensity.cpp:2103-2200
  void generate_profile_ebe(int nevent);       // :501-694
  void generate_profile_average(int nevent);   // :736-2103 (integrated-p_T entropy means)
  // events per library call (host buffers are sized for one call)
  void setBatch(int events) { batch_ = events; }
  void *context() const { return ctx_; }
  const smc_info &info() const { return info_; }

 private:
  ParameterReader *reader_;
  void *ctx_ = nullptr;
  smc_info info_{};
  smc_params params_{};
  int batch_ = 16384;
  void check(smc_status s, const char *what) const;
};

}  // namespace smc
