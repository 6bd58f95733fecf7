#include "MakeDensity.h"

#include <sys/stat.h>
#include <sys/time.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace smc {

Error::Error(smc_status s, const std::string &what) : std::runtime_error(what + ": " + smc_status_string(s)), status(s) {}

namespace {

// the values of the reference's shipped parameters.dat for the keys used here
struct Default {
  const char *name;
  double value;
};
const Default kDefaults[] = {
    {"which_mc_model", 7}, {"sub_model", 1}, {"lambda", 0.138}, {"tmax", 71}, {"tmax_subdivision", 3},
    {"alpha", 0.118}, {"Aproj", 208}, {"Atarg", 208}, {"proj_deformed", 0}, {"targ_deformed", 0},
    {"shape_of_nucleons", 2}, {"collision_criterion", 2}, {"shape_of_entropy", 2}, {"quark_width", 0.3},
    {"gauss_nucl_width", 0.812}, {"ecm", 5020.0}, {"bmin", 0.0}, {"bmax", 20.0}, {"Npmin", 2}, {"Npmax", 500},
    {"randomSeed", -1}, {"finalFactor", 40.0}, {"average_from_order", 2}, {"average_to_order", 3},
    {"ecc_from_order", 1}, {"ecc_to_order", 9}, {"use_sd", 1}, {"use_ed", 1}, {"use_4col", 0}, {"use_block", 1},
    {"maxx", 15.0}, {"maxy", 15.0}, {"dx", 0.1}, {"dy", 0.1}, {"cc_fluctuation_model", 6},
    {"cc_fluctuation_Gamma_theta", 0.75}, {"cc_fluctuation_k", 0.75}, {"generate_reaction_plane_avg_profile", 1}, {"cutdSdy", 0},
    {"cutdSdy_lowerBound", 593.51}, {"cutdSdy_upperBound", 889.53},
    {"output_TATB", 1}, {"output_rho_binary", 1}, {"output_TA", 1}, {"output_spectator_density", 1},
    // extensions (0: the reference's hard-coded value)
    {"proj_R", 0}, {"proj_a", 0}, {"targ_R", 0}, {"targ_a", 0}, {"proj_d_min", 0}, {"targ_d_min", 0},
    {"siginNN_override", 0}, {"kln_npt", 48}, {"kln_nkt", 64}, {"kln_nphi", 32}, {"max_attempts", 0},
    {"max_collisions", 0}, {"ws_inverse_cdf", 0}, {"kln_exact_band", 0},
};

double val(const ParameterReader &p, const char *name) {
  for (const Default &d : kDefaults)
    if (std::strcmp(d.name, name) == 0) return p.getVal(name, d.value);
  return p.getVal(name);
}

void ensure_data_dir() { mkdir("data", 0755); }

}  // namespace

smc_params params_from(const ParameterReader &p) {
  smc_params s{};
  s.which_mc_model = (int)val(p, "which_mc_model");
  s.sub_model = (int)val(p, "sub_model");
  s.shape_of_nucleons = (int)val(p, "shape_of_nucleons");
  s.shape_of_entropy = (int)val(p, "shape_of_entropy");
  s.collision_criterion = (int)val(p, "collision_criterion");
  s.Aproj = (int)val(p, "Aproj");
  s.Atarg = (int)val(p, "Atarg");
  s.proj_deformed = (int)val(p, "proj_deformed");
  s.targ_deformed = (int)val(p, "targ_deformed");
  s.ecm = val(p, "ecm");
  s.alpha = val(p, "alpha");
  s.gauss_nucl_width = val(p, "gauss_nucl_width");
  s.quark_width = val(p, "quark_width");
  s.lambda = val(p, "lambda");
  s.bmin = val(p, "bmin");
  s.bmax = val(p, "bmax");
  s.npmin = (int)val(p, "Npmin");
  s.npmax = (int)val(p, "Npmax");
  s.maxx = val(p, "maxx");
  s.maxy = val(p, "maxy");
  s.dx = val(p, "dx");
  s.dy = val(p, "dy");
  s.final_factor = val(p, "finalFactor");
  s.tmax = (int)val(p, "tmax");
  s.tmax_subdivision = (int)val(p, "tmax_subdivision");
  s.ecc_from_order = (int)val(p, "ecc_from_order");
  s.ecc_to_order = (int)val(p, "ecc_to_order");
  s.proj_R = val(p, "proj_R");
  s.proj_a = val(p, "proj_a");
  s.targ_R = val(p, "targ_R");
  s.targ_a = val(p, "targ_a");
  s.proj_d_min = val(p, "proj_d_min");
  s.targ_d_min = val(p, "targ_d_min");
  s.sigin_override = val(p, "siginNN_override");
  s.kln_npt = (int)val(p, "kln_npt");
  s.kln_nkt = (int)val(p, "kln_nkt");
  s.kln_nphi = (int)val(p, "kln_nphi");
  // randomSeed < 0: seeded from the clock, as src/main.cpp:27-31
  long seed = (long)val(p, "randomSeed");
  if (seed < 0) {
    timeval t;
    gettimeofday(&t, nullptr);
    seed = t.tv_usec;
  }
  s.seed = (uint64_t)seed;
  s.max_attempts = (int)val(p, "max_attempts");
  s.max_collisions = (int)val(p, "max_collisions");
  s.ws_inverse_cdf = (int)val(p, "ws_inverse_cdf");
  s.cc_fluctuation_model = (int)val(p, "cc_fluctuation_model");
  s.cc_fluctuation_gamma_theta = val(p, "cc_fluctuation_Gamma_theta");
  s.cc_fluctuation_k = val(p, "cc_fluctuation_k");
  s.kln_exact_band = val(p, "kln_exact_band");
  return s;
}

MakeDensity::MakeDensity(ParameterReader *reader) : reader_(reader) {
  params_ = params_from(*reader);
  check(smc_create(&params_, &ctx_), "smc_create");
  check(smc_get_info(ctx_, &info_), "smc_get_info");
  if (val(*reader_, "use_ed"))
    std::fprintf(stderr, "supermc_gb300: use_ed = 1: energy-density outputs (equation of state) are not produced\n");
}

MakeDensity::~MakeDensity() { smc_destroy(ctx_); }

void MakeDensity::check(smc_status s, const char *what) const {
  if (s != SMC_OK) throw Error(s, what);
}

void MakeDensity::generateEccTable(int nevent) {
  ensure_data_dir();
  const int from = (int)val(*reader_, "ecc_from_order"), to = (int)val(*reader_, "ecc_to_order");
  const bool sd = val(*reader_, "use_sd") != 0;
  // dumpEccentricities' deformed layout (src/MakeDensity.cpp:2249-2251)
  const bool deformed = val(*reader_, "proj_deformed") == 1 || val(*reader_, "targ_deformed") == 1;
  std::vector<double> ecc, ori;
  for (int done = 0; done < nevent; done += batch_) {
    const int n = std::min(batch_, nevent - done);
    ecc.resize((size_t)n * 49);
    ori.resize((size_t)n * 4);
    smc_outputs out{};
    out.ecc = ecc.data();
    if (deformed) out.orientation = ori.data();
    check(smc_generate(ctx_, (uint64_t)done, n, &out), "smc_generate");
    if (sd && deformed)
      check(smc_write_ecc_deformed(ecc.data(), ori.data(), n, from, to, "data/sn_ecc_eccp_%d.dat"),
            "smc_write_ecc_deformed");
    else if (sd)
      check(smc_write_ecc(ecc.data(), n, from, to, "data/sn_ecc_eccp_%d.dat"), "smc_write_ecc");
  }
}

void MakeDensity::generate_profile_ebe(int nevent) {
  ensure_data_dir();
  const bool sd = val(*reader_, "use_sd") != 0, block = val(*reader_, "use_block") != 0,
             four = val(*reader_, "use_4col") != 0;
  // cutdSdy: an event whose dS/dy = sum getRho dx dy lies outside
  // [cutdSdy_lowerBound, cutdSdy_upperBound] is dropped after its pairing
  // (its binary.dat lines stay) and does not count (src/MakeDensity.cpp:
  // 601-617, :683-684, gettotaldSdy :2557-2567)
  const bool cut = val(*reader_, "cutdSdy") == 1;
  const double cut_lo = val(*reader_, "cutdSdy_lowerBound"), cut_hi = val(*reader_, "cutdSdy_upperBound");
  const double ff = params_.final_factor, area = params_.dx * params_.dy;
  const size_t g = (size_t)info_.nx * info_.ny;
  const int AB = info_.A + info_.B, mc = info_.max_collisions;
  const int batch = std::max(1, std::min(batch_, 1024));   // host grids of one call
  std::vector<float> rho;
  std::vector<int> npart, ncoll;
  std::vector<double> grid(g), pos, coll;
  std::vector<uint8_t> wounded;
  char name[256];
  int event = 0;                 // events written
  uint64_t generated = 0;        // event ids used
  while (event < nevent) {
    const int n = std::min(batch, cut ? batch : nevent - event);
    rho.resize((size_t)n * g);
    npart.resize((size_t)n * 2);
    ncoll.resize(n);
    pos.resize((size_t)n * AB * 2);
    wounded.resize((size_t)n * AB);
    coll.resize((size_t)n * mc * 2);
    smc_outputs out{};
    out.rho = rho.data();
    out.npart = npart.data();
    out.ncoll = ncoll.data();
    out.positions = pos.data();
    out.wounded = wounded.data();
    out.collisions = coll.data();
    check(smc_generate(ctx_, generated, n, &out), "smc_generate");
    generated += n;
    for (int e = 0; e < n && event < nevent; e++) {
      // MCnucl::dumpBinaryTable("data/binary.dat") after each event's pairing
      // (src/MakeDensity.cpp:598; src/MCnucl.cpp:1175-1207)
      check(smc_write_binary_table(coll.data() + (size_t)e * mc * 2, std::min(ncoll[e], mc), "data/binary.dat"),
            "smc_write_binary_table");
      if (cut) {
        double total = 0.0;
        for (size_t k = 0; k < g; k++) total += (double)rho[(size_t)e * g + k] * area;
        if (total < cut_lo || total > cut_hi) continue;
      }
      event++;
      if (event == nevent)
        check(smc_write_nucleon_tables(pos.data() + (size_t)e * AB * 2, wounded.data() + (size_t)e * AB, info_.A,
                                       info_.B, "data/wounded.data", "data/nucl1.data", "data/nucl2.data"),
              "smc_write_nucleon_tables");
      if (!sd) continue;
      // MakeDensity::setSd (src/MakeDensity.cpp:2514-2522)
      for (size_t k = 0; k < g; k++) grid[k] = (double)rho[(size_t)e * g + k] * ff;
      if (four) {
        std::snprintf(name, sizeof(name), "data/sd_event_%d_4col.dat", event);
        check(smc_write_density_4col(grid.data(), info_.nx, info_.ny, -params_.maxx, -params_.maxy, params_.dx,
                                     params_.dy, 0.0, (double)(npart[2 * e] + npart[2 * e + 1]), name),
              "smc_write_density_4col");
      }
      if (block) {
        std::snprintf(name, sizeof(name), "data/sd_event_%d_block.dat", event);
        check(smc_write_density_block(grid.data(), info_.nx, info_.ny, name), "smc_write_density_block");
      }
    }
  }
}

void MakeDensity::generate_profile_average(int nevent) {
  ensure_data_dir();
  const int from = (int)val(*reader_, "average_from_order"), to = (int)val(*reader_, "average_to_order");
  const bool sd = val(*reader_, "use_sd") != 0, block = val(*reader_, "use_block") != 0,
             four = val(*reader_, "use_4col") != 0;
  const bool rp = val(*reader_, "generate_reaction_plane_avg_profile") == 1;
  const bool tatb = val(*reader_, "output_TATB") != 0, rhob = val(*reader_, "output_rho_binary") != 0,
             ta = val(*reader_, "output_TA") != 0, spect = val(*reader_, "output_spectator_density") != 0;
  const bool thick_ok = params_.which_mc_model != 7;   // sqrt(T_A T_B) has no thickness planes here
  if ((tatb || ta) && !thick_ok)
    std::fprintf(stderr, "supermc_gb300: output_TATB / output_TA: not produced for which_mc_model 7\n");
  const size_t g = (size_t)info_.nx * info_.ny;
  const int no = to - from + 1;
  // grids, in the order of smc_average_outputs
  std::vector<double> grid[14];
  smc_average_outputs o{};
  double **slot[14] = {&o.sd, &o.sd_rp, &o.ta_tb, &o.ta_tb_rp, &o.ta, &o.tb, &o.ta_rp, &o.tb_rp,
                       &o.rho_binary, &o.rho_binary_rp, &o.spectator_a, &o.spectator_b, &o.spectator_a_rp,
                       &o.spectator_b_rp};
  const bool on[14] = {true, rp, tatb && thick_ok, tatb && thick_ok && rp, ta && thick_ok, ta && thick_ok,
                       ta && thick_ok && rp, ta && thick_ok && rp, rhob, rhob && rp, spect, spect, false, false};
  // file stems (MakeDensity.cpp:741-1180; the reference writes no spectator
  // means in the reaction-plane frame)
  const char *stem[14] = {"sdAvg_order", "sdAvg_RP_order", "TATB_fromSd_order", "TATB_fromSd_RP_order",
                          "nuclear_thickness_TA_fromSd_order", "nuclear_thickness_TB_fromSd_order",
                          "nuclear_thickness_TA_fromSd_RP_order", "nuclear_thickness_TB_fromSd_RP_order",
                          "rho_binary_fromSd_order", "rho_binary_fromSd_RP_order",
                          "spectator_density_A_fromSd_order", "spectator_density_B_fromSd_order", "", ""};
  for (int k = 0; k < 14; k++)
    if (on[k]) {
      grid[k].assign(g * no, 0.0);
      *slot[k] = grid[k].data();
    }
  int used = 0;
  check(smc_average_profiles(ctx_, 0, nevent, nullptr, nullptr, nullptr, from, to, &o, &used),
        "smc_average_profiles");
  if (!sd) return;
  char name[256];
  for (int k = 0; k < 14; k++) {
    if (!on[k]) continue;
    for (int q = 0; q < no; q++) {
      const double *m = grid[k].data() + (size_t)q * g;
      const int order = from + q;
      if (four) {
        std::snprintf(name, sizeof(name), "data/%s_%d_4col.dat", stem[k], order);
        check(smc_write_density_4col(m, info_.nx, info_.ny, -params_.maxx, -params_.maxy, params_.dx, params_.dy,
                                     0.0, 0.0, name),
              "smc_write_density_4col");
      }
      if (block) {
        std::snprintf(name, sizeof(name), "data/%s_%d_block.dat", stem[k], order);
        check(smc_write_density_block(m, info_.nx, info_.ny, name), "smc_write_density_block");
      }
    }
  }
}

}  // namespace smc
