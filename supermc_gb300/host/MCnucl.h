// The reference's MCnucl call surface (src/MCnucl.h:85-140) over the GPU
// library's C ABI (include/supermc.h), one event at a time, for code written
// against MCnucl:
//   MCnucl mc(&reader);
//   mc.generateNuclei(b);                  // src/MCnucl.cpp:208-214
//   if (mc.getBinaryCollision() && mc.CentralityCut()) {   // :217-308, :388-393
//     mc.calculateThickness();             // :398-478
//     mc.setDensity(0, -1);                // :626-866
//     ... mc.getTA1(i, j), mc.getRho(0, i, j) ...
//     mc.rotateGrid(0, 2); mc.calculateThickness(); mc.setDensity(0, -1);   // :1152-1174
//   }
//   mc.deleteNucleus();
// Each generateNuclei draws a new event from the context's Philox streams
// (the event ids count up from 0; the reference draws from drand48).  The
// grids are the library's FP32 grids read back to the host.  In a moved
// frame (recenterGrid / rotateGrid) the event's sequence of moves is the
// reference's averaged-mode sequence (src/MakeDensity.cpp:1289-1334: for each
// order, recenterGrid then rotateGrid, the orders increasing), which the
// library runs as one call.  Only the p_T-integrated density (ipt < 0).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/supermc.h"
#include "MakeDensity.h"
#include "ParameterReader.h"

namespace smc {

class MCnucl {
 public:
  explicit MCnucl(ParameterReader *reader);   // src/MCnucl.cpp:22-154 (MC-KLN: the dN/dy table too)
  ~MCnucl();
  MCnucl(const MCnucl &) = delete;
  MCnucl &operator=(const MCnucl &) = delete;

  // orientations (cos theta, phi) of the projectile and the target drawn by
  // the last generateNuclei (src/MCnucl.h:90; the reference never sets them)
  double lastCx1 = 0, lastPh1 = 0, lastCx2 = 0, lastPh2 = 0;

  void generateNuclei(double b);
  void deleteNucleus();
  int getBinaryCollision();                    // the number of binary collisions
  int CentralityCut();                         // 1: Npmin <= Npart1 + Npart2 <= Npmax
  void setCentralityCut(int Nmin, int Nmax) { npmin_ = Nmin; npmax_ = Nmax; }
  void calculateThickness();
  void setDensity(int iy, int ipt);            // ipt < 0 only (the p_T-integrated density)
  void recenterGrid(int iy, int n = 2);
  void rotateGrid(int iy, int n = 2);
  void makeTable() {}                          // built by the constructor (MC-KLN)

  double getTA1(int x, int y) const { return ta_[(size_t)x * info_.ny + y]; }
  double getTA2(int x, int y) const { return tb_[(size_t)x * info_.ny + y]; }
  double getRho(int iy, int x, int y) const { (void)iy; return rho_[(size_t)x * info_.ny + y]; }
  int getNcoll() const { return ncoll_; }
  int getNpart1() const { return npart_[0]; }
  int getNpart2() const { return npart_[1]; }
  double getdNdy() const;                      // sum getRho dx dy (src/MCnucl.h:100-104)

  void dumpBinaryTable(const std::string &filename);       // src/MCnucl.cpp:1175-1189
  void dumpparticipantTable(const std::string &filename);  // :1193-1207

  // the current nuclei: x, y of every nucleon (sorted by x) and the impact parameter
  const std::vector<double> &projectile() const { return xy_proj_; }
  const std::vector<double> &target() const { return xy_targ_; }
  double impactParameter() const { return b_; }
  const smc_info &info() const { return info_; }

 private:
  enum class Frame { Lab, ReactionPlane, ParticipantPlane };
  void check(smc_status s, const char *what) const;
  void inject(bool thickness, bool density);
  void moved(bool thickness, bool density);

  void *ctx_ = nullptr;
  smc_params params_{};
  smc_info info_{};
  int npmin_ = 0, npmax_ = 0;
  uint64_t next_event_ = 0;
  bool have_ = false;
  double b_ = 0;
  std::vector<double> xy_proj_, xy_targ_;
  int npart_[2] = {0, 0}, ncoll_ = 0;
  std::vector<float> ta_, tb_, rho_;
  Frame frame_ = Frame::Lab;
  int from_order_ = 0, order_ = 0;   // the moves so far: orders from_order_ .. order_
};

}  // namespace smc
