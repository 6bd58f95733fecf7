#include "MCnucl.h"

#include <algorithm>

namespace smc {

MCnucl::MCnucl(ParameterReader *reader) {
  params_ = params_from(*reader);
  check(smc_create(&params_, &ctx_), "smc_create");
  try {
    load_light_tables(ctx_, params_);
  } catch (...) {
    smc_destroy(ctx_);
    throw;
  }
  check(smc_get_info(ctx_, &info_), "smc_get_info");
  npmin_ = params_.npmin;
  npmax_ = params_.npmax;
  const size_t g = (size_t)info_.nx * info_.ny;
  ta_.assign(g, 0.f);
  tb_.assign(g, 0.f);
  rho_.assign(g, 0.f);
}

MCnucl::~MCnucl() { smc_destroy(ctx_); }

void MCnucl::check(smc_status s, const char *what) const {
  if (s != SMC_OK) throw Error(s, what);
}

void MCnucl::generateNuclei(double b) {
  xy_proj_.assign((size_t)2 * info_.A, 0.0);
  xy_targ_.assign((size_t)2 * info_.B, 0.0);
  double ori[4];
  check(smc_sample_nuclei(ctx_, next_event_++, b, xy_proj_.data(), xy_targ_.data(), npart_, &ncoll_, ori),
        "smc_sample_nuclei");
  lastCx1 = ori[0]; lastPh1 = ori[1]; lastCx2 = ori[2]; lastPh2 = ori[3];
  b_ = b;
  have_ = true;
  frame_ = Frame::Lab;
  from_order_ = order_ = 0;
  std::fill(ta_.begin(), ta_.end(), 0.f);
  std::fill(tb_.begin(), tb_.end(), 0.f);
  std::fill(rho_.begin(), rho_.end(), 0.f);
}

void MCnucl::deleteNucleus() {
  have_ = false;
  xy_proj_.clear();
  xy_targ_.clear();
  npart_[0] = npart_[1] = ncoll_ = 0;
  frame_ = Frame::Lab;
}

int MCnucl::getBinaryCollision() {
  if (!have_) throw Error(SMC_ERR_ARGUMENT, "getBinaryCollision: no nuclei (generateNuclei)");
  return ncoll_;
}

int MCnucl::CentralityCut() {
  const int np = npart_[0] + npart_[1];
  return (np <= npmax_ && np >= npmin_) ? 1 : 0;
}

// the current event through smc_inject: T_A, T_B (when the model makes
// them) and the density
void MCnucl::inject(bool thickness, bool density) {
  if (!have_) throw Error(SMC_ERR_ARGUMENT, "no nuclei (generateNuclei)");
  smc_outputs out{};
  if (thickness && params_.which_mc_model != 7) {
    out.ta = ta_.data();
    out.tb = tb_.data();
  }
  if (density || thickness) out.rho = rho_.data();
  check(smc_inject(ctx_, 1, xy_proj_.data(), xy_targ_.data(), &b_, &out), "smc_inject");
}

// the current event after its moves (orders from_order_ .. order_, the
// reference's averaged-mode sequence): the grids of the last move's frame
void MCnucl::moved(bool thickness, bool density) {
  if (!have_) throw Error(SMC_ERR_ARGUMENT, "no nuclei (generateNuclei)");
  const size_t g = (size_t)info_.nx * info_.ny;
  const int no = order_ - from_order_ + 1;
  std::vector<double> sd((size_t)no * g), ta, tb;
  smc_average_outputs out{};
  const bool rp = frame_ == Frame::ReactionPlane;
  (rp ? out.sd_rp : out.sd) = sd.data();
  if (thickness && params_.which_mc_model != 7) {
    ta.assign((size_t)no * g, 0.0);
    tb.assign((size_t)no * g, 0.0);
    (rp ? out.ta_rp : out.ta) = ta.data();
    (rp ? out.tb_rp : out.tb) = tb.data();
  }
  int used = 0;
  check(smc_average_profiles(ctx_, 0, 1, xy_proj_.data(), xy_targ_.data(), &b_, from_order_, order_, &out, &used),
        "smc_average_profiles");
  const size_t last = (size_t)(no - 1) * g;
  const double ff = params_.final_factor;
  for (size_t k = 0; k < g; k++) {
    rho_[k] = used ? (float)(sd[last + k] / ff) : 0.f;
    if (!ta.empty()) {
      ta_[k] = used ? (float)ta[last + k] : 0.f;
      tb_[k] = used ? (float)tb[last + k] : 0.f;
    }
  }
  (void)density;
}

void MCnucl::calculateThickness() {
  if (frame_ == Frame::Lab) inject(true, true);
  else moved(true, true);
}

void MCnucl::setDensity(int iy, int ipt) {
  (void)iy;
  if (ipt >= 0) throw Error(SMC_ERR_CONFIG, "setDensity: only the p_T-integrated density (ipt < 0)");
  if (frame_ == Frame::Lab) inject(false, true);
  else moved(false, true);
}

void MCnucl::recenterGrid(int iy, int n) {
  (void)iy;
  if (frame_ == Frame::Lab) from_order_ = n;
  else if (n < order_ || (n == order_ && frame_ == Frame::ParticipantPlane))
    throw Error(SMC_ERR_ARGUMENT, "recenterGrid: moves follow the averaged-mode sequence (increasing orders)");
  order_ = n;
  frame_ = Frame::ReactionPlane;
}

void MCnucl::rotateGrid(int iy, int n) {
  (void)iy;
  if (frame_ == Frame::Lab) from_order_ = n;
  else if (n < order_ || (n == order_ && frame_ == Frame::ParticipantPlane))
    throw Error(SMC_ERR_ARGUMENT, "rotateGrid: moves follow the averaged-mode sequence (increasing orders)");
  order_ = n;
  frame_ = Frame::ParticipantPlane;
}

double MCnucl::getdNdy() const {
  double s = 0.0;
  for (float v : rho_) s += v;
  return s * params_.dx * params_.dy;
}

void MCnucl::dumpBinaryTable(const std::string &filename) {
  if (!have_) throw Error(SMC_ERR_ARGUMENT, "dumpBinaryTable: no nuclei (generateNuclei)");
  const int AB = info_.A + info_.B;
  std::vector<double> coll((size_t)2 * info_.max_collisions), pos((size_t)2 * AB);
  std::vector<uint8_t> wounded(AB);
  smc_outputs out{};
  out.collisions = coll.data();
  out.positions = pos.data();
  out.wounded = wounded.data();
  check(smc_inject(ctx_, 1, xy_proj_.data(), xy_targ_.data(), &b_, &out), "smc_inject");
  check(smc_write_binary_table(coll.data(), std::min(ncoll_, info_.max_collisions), filename.c_str()),
        "smc_write_binary_table");
  // the reference's dumpBinaryTable also rewrites these (src/MCnucl.cpp:1191-1207)
  check(smc_write_nucleon_tables(pos.data(), wounded.data(), info_.A, info_.B, "data/wounded.data",
                                 "data/nucl1.data", "data/nucl2.data"),
        "smc_write_nucleon_tables");
}

void MCnucl::dumpparticipantTable(const std::string &filename) {
  if (!have_) throw Error(SMC_ERR_ARGUMENT, "dumpparticipantTable: no nuclei (generateNuclei)");
  const int AB = info_.A + info_.B;
  std::vector<double> pos((size_t)2 * AB);
  std::vector<uint8_t> wounded(AB);
  smc_outputs out{};
  out.positions = pos.data();
  out.wounded = wounded.data();
  check(smc_inject(ctx_, 1, xy_proj_.data(), xy_targ_.data(), &b_, &out), "smc_inject");
  check(smc_write_nucleon_tables(pos.data(), wounded.data(), info_.A, info_.B, filename.c_str(), nullptr, nullptr),
        "smc_write_nucleon_tables");
}

}  // namespace smc
