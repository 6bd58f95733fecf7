#include "MakeDensity.h"

#include <sys/stat.h>
#include <sys/time.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace smc {

Error::Error(smc_status s, const std::string &what)
    : std::runtime_error(what + ": " + smc_status_string(s) +
                         (s == SMC_ERR_CUDA ? std::string(" (") + smc_cuda_error_string() + ")" : std::string())),
      status(s) {}

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
    {"output_rhob", 0}, {"PT_flag", 1}, {"mixedMode", 0}, {"PT_Min", 0.1}, {"PT_Max", 2}, {"d_PT", 0.1},
    {"use_5col", 0}, {"use_ptCol", 0},
    // extensions (0: the reference's hard-coded value)
    {"proj_R", 0}, {"proj_a", 0}, {"targ_R", 0}, {"targ_a", 0}, {"proj_d_min", 0}, {"targ_d_min", 0},
    {"siginNN_override", 0}, {"kln_npt", 48}, {"kln_nkt", 64}, {"kln_nphi", 32}, {"max_attempts", 0},
    {"max_collisions", 0}, {"ws_inverse_cdf", 0}, {"kln_exact_band", 0}, {"use_binary", 0},
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

void load_light_tables(void *ctx, const smc_params &p) {
  const int masses[2] = {p.Aproj, p.Atarg};
  for (int w = 0; w < 2; w++) {
    const int A = masses[w];
    const char *file = A == 3 ? "tables/he3_plaintext.dat" : A == 4 ? "tables/he4_plaintext.dat"
                     : A == 12 ? "tables/carbon_plaintext.dat" : A == 16 ? "tables/oxygen_plaintext.dat" : nullptr;
    if (!file || (w == 1 && A == masses[0])) continue;   // one table per mass number
    smc_status s = smc_load_configurations(ctx, A, file);
    if (s != SMC_OK) throw Error(s, std::string("Error: ") + file + " does not find (or holds no configuration)");
  }
}

MakeDensity::MakeDensity(ParameterReader *reader) : reader_(reader) {
  params_ = params_from(*reader);
  check(smc_create(&params_, &ctx_), "smc_create");
  try {
    load_light_tables(ctx_, params_);
  } catch (...) {
    smc_destroy(ctx_);
    throw;
  }
  check(smc_get_info(ctx_, &info_), "smc_get_info");
  binary_ = val(*reader_, "use_binary") == 1;
  if (val(*reader_, "use_ed"))
    std::fprintf(stderr, "supermc_gb300: use_ed = 1: energy-density outputs (equation of state) are not produced\n");
}

MakeDensity::~MakeDensity() { smc_destroy(ctx_); }

void MakeDensity::check(smc_status s, const char *what) const {
  if (s != SMC_OK) throw Error(s, what);
}

namespace {

// use_binary = 1: each table goes to a NumPy .npy file of the same name in
// place of the text file, with the text file's columns at full precision
void write_block(const double *grid, int nx, int ny, const char *stem, bool binary) {
  char name[512];
  std::snprintf(name, sizeof(name), "%s_block.%s", stem, binary ? "npy" : "dat");
  if (binary) {
    const int64_t shape[2] = {nx, ny};
    MakeDensity::check_status(smc_write_npy(name, grid, 8, 2, shape, 0), "smc_write_npy");
  } else {
    MakeDensity::check_status(smc_write_density_block(grid, nx, ny, name), "smc_write_density_block");
  }
}

void write_4col(const double *grid, int nx, int ny, const smc_params &p, double npart, const char *stem,
                bool binary) {
  char name[512];
  std::snprintf(name, sizeof(name), "%s_4col.%s", stem, binary ? "npy" : "dat");
  if (!binary) {
    MakeDensity::check_status(
        smc_write_density_4col(grid, nx, ny, -p.maxx, -p.maxy, p.dx, p.dy, 0.0, npart, name),
        "smc_write_density_4col");
    return;
  }
  std::vector<double> rows((size_t)nx * ny * 4);
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double *r = rows.data() + ((size_t)i * ny + j) * 4;
      r[0] = 0.0;
      r[1] = -p.maxx + i * p.dx;
      r[2] = -p.maxy + j * p.dy;
      r[3] = grid[(size_t)i * ny + j];
    }
  const int64_t shape[2] = {(int64_t)nx * ny, 4};
  MakeDensity::check_status(smc_write_npy(name, rows.data(), 8, 2, shape, 0), "smc_write_npy");
}

}  // namespace

void MakeDensity::check_status(smc_status s, const char *what) {
  if (s != SMC_OK) throw Error(s, what);
}

void MakeDensity::setSd(const float *rho, double *sd) const {
  const size_t g = (size_t)info_.nx * info_.ny;
  for (size_t k = 0; k < g; k++) sd[k] = (double)rho[k] * params_.final_factor;
}

double MakeDensity::gettotaldSdy(const float *rho) const {
  const size_t g = (size_t)info_.nx * info_.ny;
  double sum = 0.0;
  for (size_t k = 0; k < g; k++) sum += (double)rho[k] * params_.dx * params_.dy;
  return sum;
}

void MakeDensity::dumpDensityBlock(const char *filename, const double *grid) const {
  check(smc_write_density_block(grid, info_.nx, info_.ny, filename), "smc_write_density_block");
}

void MakeDensity::dumpDensity4Col(const char *filename, const double *grid, double npart) const {
  check(smc_write_density_4col(grid, info_.nx, info_.ny, -params_.maxx, -params_.maxy, params_.dx, params_.dy, 0.0,
                               npart, filename),
        "smc_write_density_4col");
}

void MakeDensity::dumpEccentricities(const char *base_filename, const double *ecc, int n, int from_order,
                                     int to_order, const double *orientation) const {
  if (!base_filename) throw Error(SMC_ERR_ARGUMENT, "dumpEccentricities: no file name");
  std::string pattern;
  for (const char *c = base_filename; *c; c++) {
    pattern += *c;
    if (*c == '%') pattern += '%';   // a literal '%' of the name
  }
  pattern += "_%d.dat";
  if (orientation)
    check(smc_write_ecc_deformed(ecc, orientation, n, from_order, to_order, pattern.c_str()),
          "smc_write_ecc_deformed");
  else
    check(smc_write_ecc(ecc, n, from_order, to_order, pattern.c_str()), "smc_write_ecc");
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
    if (sd && binary_)
      check(smc_write_ecc_npy(ecc.data(), deformed ? ori.data() : nullptr, n, from, to, "data/sn_ecc_eccp_%d.npy"),
            "smc_write_ecc_npy");
    else if (sd && deformed)
      check(smc_write_ecc_deformed(ecc.data(), ori.data(), n, from, to, "data/sn_ecc_eccp_%d.dat"),
            "smc_write_ecc_deformed");
    else if (sd)
      check(smc_write_ecc(ecc.data(), n, from, to, "data/sn_ecc_eccp_%d.dat"), "smc_write_ecc");
  }
}

// wounded.data / nucl1.data / nucl2.data as .npy: participants [k][3]
// (x, y, nucleus 1 or 2), projectile [A][2], target [B][2]
void MakeDensity::write_nucleon_npy(const double *xy, const uint8_t *wounded) {
  const int A = info_.A, B = info_.B;
  std::vector<double> part;
  for (int k = 0; k < A + B; k++)
    if (wounded[k]) part.insert(part.end(), {xy[2 * k], xy[2 * k + 1], k < A ? 1.0 : 2.0});
  const int64_t sp[2] = {(int64_t)(part.size() / 3), 3}, s1[2] = {A, 2}, s2[2] = {B, 2};
  check(smc_write_npy("data/wounded.npy", part.data(), 8, 2, sp, 0), "smc_write_npy");
  check(smc_write_npy("data/nucl1.npy", xy, 8, 2, s1, 0), "smc_write_npy");
  check(smc_write_npy("data/nucl2.npy", xy + 2 * (size_t)A, 8, 2, s2, 0), "smc_write_npy");
}

void MakeDensity::generate_profile_ebe(int nevent) {
  ensure_data_dir();
  const bool sd = val(*reader_, "use_sd") != 0, block = val(*reader_, "use_block") != 0,
             four = val(*reader_, "use_4col") != 0;
  // cutdSdy: an event whose dS/dy = sum getRho dx dy lies outside
  // [cutdSdy_lowerBound, cutdSdy_upperBound] is dropped after its pairing
  // (its binary.dat lines stay) and does not count (src/MakeDensity.cpp:
  // 601-617, :683-684, gettotaldSdy :2557-2567)
  // PT_flag > 0: the p_T-integrated profiles; PT_flag < 0 or mixedMode > 0:
  // the p_T-differential ones of MC-KLN as well (MakeDensity::MakeDensity,
  // src/MakeDensity.cpp:106-119; :563-688).  Their files are written when
  // use_5col / use_ptCol are set: the reference reads those switches into
  // locals that shadow the ones it tests (:556-567), so its operation 1
  // writes none.  The cut on dS/dy applies with PT_flag > 0 only (:604-617).
  const bool pt_inte = val(*reader_, "PT_flag") > 0;
  const bool want_pt = (!pt_inte || val(*reader_, "mixedMode") > 0) && params_.which_mc_model == 1;
  const bool five = val(*reader_, "use_5col") != 0, ptcol = val(*reader_, "use_ptCol") != 0;
  int nbins = 0;
  if (want_pt) {
    const double ptmin = val(*reader_, "PT_Min"), ptmax = val(*reader_, "PT_Max"), dpt = val(*reader_, "d_PT");
    nbins = (int)((ptmax - ptmin) / dpt + 0.1) + 1;   // MaxPT, src/MakeDensity.cpp:71
    check(smc_kln_pt_table(ctx_, ptmin, dpt, nbins, nullptr, 0), "smc_kln_pt_table");
  }
  const bool cut = val(*reader_, "cutdSdy") == 1 && pt_inte;
  const double cut_lo = val(*reader_, "cutdSdy_lowerBound"), cut_hi = val(*reader_, "cutdSdy_upperBound");
  const double ff = params_.final_factor, area = params_.dx * params_.dy;
  const size_t g = (size_t)info_.nx * info_.ny;
  const int AB = info_.A + info_.B, mc = info_.max_collisions;
  // host grids of one call (the p_T-differential ones hold nbins per cell)
  const int batch = std::max(1, std::min(batch_, want_pt ? 32 : 1024));
  std::vector<float> rho, rho_pt;
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
    if (want_pt) {
      rho_pt.resize((size_t)n * g * nbins);
      out.rho_pt = rho_pt.data();
    }
    check(smc_generate(ctx_, generated, n, &out), "smc_generate");
    generated += n;
    for (int e = 0; e < n && event < nevent; e++) {
      // MCnucl::dumpBinaryTable("data/binary.dat") after each event's pairing
      // (src/MakeDensity.cpp:598; src/MCnucl.cpp:1175-1207)
      const int nc = std::min(ncoll[e], mc);
      if (binary_) {
        const int64_t shape[2] = {nc, 2};
        check(smc_write_npy("data/binary.npy", coll.data() + (size_t)e * mc * 2, 8, 2, shape, 1), "smc_write_npy");
      } else {
        check(smc_write_binary_table(coll.data() + (size_t)e * mc * 2, nc, "data/binary.dat"),
              "smc_write_binary_table");
      }
      if (cut) {
        double total = 0.0;
        for (size_t k = 0; k < g; k++) total += (double)rho[(size_t)e * g + k] * area;
        if (total < cut_lo || total > cut_hi) continue;
      }
      event++;
      if (event == nevent && binary_)
        write_nucleon_npy(pos.data() + (size_t)e * AB * 2, wounded.data() + (size_t)e * AB);
      else if (event == nevent)
        check(smc_write_nucleon_tables(pos.data() + (size_t)e * AB * 2, wounded.data() + (size_t)e * AB, info_.A,
                                       info_.B, "data/wounded.data", "data/nucl1.data", "data/nucl2.data"),
              "smc_write_nucleon_tables");
      if (!sd) continue;
      const double np = (double)(npart[2 * e] + npart[2 * e + 1]);
      if (want_pt && (five || ptcol)) {   // setSd of the p_T bins, dumpDensity5Col / dumpDesityptCol
        const float *d = rho_pt.data() + (size_t)e * g * nbins;
        if (five) {
          std::snprintf(name, sizeof(name), "data/sd_event_%d_5col.dat", event);
          check(smc_write_density_pt(d, info_.nx, info_.ny, nbins, np, ff, name), "smc_write_density_pt");
        }
        if (ptcol) {
          std::snprintf(name, sizeof(name), "data/sd_event_%d_ptCol.dat", event);
          check(smc_write_density_pt(d, info_.nx, info_.ny, nbins, np, ff, name), "smc_write_density_pt");
        }
      }
      if (!pt_inte) continue;
      // MakeDensity::setSd (src/MakeDensity.cpp:2514-2522)
      for (size_t k = 0; k < g; k++) grid[k] = (double)rho[(size_t)e * g + k] * ff;
      std::snprintf(name, sizeof(name), "data/sd_event_%d", event);
      if (four) write_4col(grid.data(), info_.nx, info_.ny, params_, np, name, binary_);
      if (block) write_block(grid.data(), info_.nx, info_.ny, name, binary_);
    }
  }
}

void MakeDensity::generate_profile_ebe_Jet(int nevent) {
  // the reference's constructor exits for operation 2 with PT_flag < 0
  // (src/MakeDensity.cpp:121-131)
  if (val(*reader_, "PT_flag") < 0)
    throw Error(SMC_ERR_CONFIG, "This option is not supported: Operation=2, PTinte<0");
  ensure_data_dir();
  const int from = (int)val(*reader_, "ecc_from_order"), to = (int)val(*reader_, "ecc_to_order");
  const bool sd = val(*reader_, "use_sd") != 0, block = val(*reader_, "use_block") != 0,
             four = val(*reader_, "use_4col") != 0;
  const bool rhob_on = val(*reader_, "output_rho_binary") != 0, ta_on = val(*reader_, "output_TA") != 0,
             nb_on = val(*reader_, "output_rhob") != 0, spect_on = val(*reader_, "output_spectator_density") != 0;
  const bool thick_ok = params_.which_mc_model != 7;   // sqrt(T_A T_B) has no thickness planes here
  if ((ta_on || nb_on) && !thick_ok)
    std::fprintf(stderr, "supermc_gb300: output_TA / output_rhob: not produced for which_mc_model 7\n");
  const bool deformed = val(*reader_, "proj_deformed") == 1 || val(*reader_, "targ_deformed") == 1;
  const bool cut = val(*reader_, "cutdSdy") == 1;
  const double cut_lo = val(*reader_, "cutdSdy_lowerBound"), cut_hi = val(*reader_, "cutdSdy_upperBound");
  const double ff = params_.final_factor, area = params_.dx * params_.dy;
  const size_t g = (size_t)info_.nx * info_.ny;
  const int A = info_.A, B = info_.B, AB = A + B, mc = info_.max_collisions;
  const int batch = std::max(1, std::min(batch_, 256));   // host grids of one call
  const bool want_t = (ta_on || nb_on) && thick_ok;
  std::vector<float> rho, ta, tb, rb, spa, spb;
  std::vector<int> npart, ncoll;
  std::vector<double> grid(g), pos, coll, ecc, ori;
  std::vector<uint8_t> wounded;
  char name[256], pattern[256];
  int event = 1;                 // the event number of the files (events that passed the cut + 1)
  uint64_t generated = 0;        // event ids used
  while (event <= nevent) {
    const int n = std::min(batch, cut ? batch : nevent - event + 1);
    rho.resize((size_t)n * g);
    npart.resize((size_t)n * 2);
    ncoll.resize(n);
    pos.resize((size_t)n * AB * 2);
    wounded.resize((size_t)n * AB);
    coll.resize((size_t)n * mc * 2);
    ecc.resize((size_t)n * 49);
    ori.resize((size_t)n * 4);
    smc_outputs out{};
    out.rho = rho.data();
    out.ecc = ecc.data();
    out.npart = npart.data();
    out.ncoll = ncoll.data();
    out.positions = pos.data();
    out.wounded = wounded.data();
    out.collisions = coll.data();
    if (deformed) out.orientation = ori.data();
    if (want_t) {
      ta.resize((size_t)n * g);
      tb.resize((size_t)n * g);
      out.ta = ta.data();
      out.tb = tb.data();
    }
    if (rhob_on) {
      rb.resize((size_t)n * g);
      out.rho_binary = rb.data();
    }
    if (spect_on) {
      spa.resize((size_t)n * g);
      spb.resize((size_t)n * g);
      out.spectator_a = spa.data();
      out.spectator_b = spb.data();
    }
    check(smc_generate(ctx_, generated, n, &out), "smc_generate");
    generated += n;
    for (int e = 0; e < n && event <= nevent; e++) {
      const double *xy = pos.data() + (size_t)e * AB * 2;
      const uint8_t *wd = wounded.data() + (size_t)e * AB;
      const double np = (double)(npart[2 * e] + npart[2 * e + 1]);
      // the event's tables, written after its pairing whatever the cut
      // decides (src/MakeDensity.cpp:299-305); an event that fails the cut
      // leaves them under the number the next event reuses
      std::snprintf(name, sizeof(name), "data/ParticipantTable_event_%d.dat", event);
      check(smc_write_participant_table(xy, wd, A, B, name), "smc_write_participant_table");
      std::snprintf(name, sizeof(name), "data/Spectators_event_%d.dat", event);
      check(smc_write_spectator_table(xy, wd, A, B, params_.ecm, name), "smc_write_spectator_table");
      std::snprintf(name, sizeof(name), "data/BinaryCollisionTable_event_%d.dat", event);
      const int nc = std::min(ncoll[e], mc);
      check(smc_write_binary_table(coll.data() + (size_t)e * mc * 2, nc, name), "smc_write_binary_table");
      // MCnucl::dumpBinaryTable also rewrites the nucleon tables (src/MCnucl.cpp:1191-1207)
      check(smc_write_nucleon_tables(xy, wd, A, B, "data/wounded.data", "data/nucl1.data", "data/nucl2.data"),
            "smc_write_nucleon_tables");
      if (cut) {
        double total = 0.0;
        for (size_t k = 0; k < g; k++) total += (double)rho[(size_t)e * g + k] * area;
        if (total < cut_lo || total > cut_hi) continue;
      }
      auto grids = [&](const float *src, double scale, const char *stem_fmt) {
        for (size_t k = 0; k < g; k++) grid[k] = (double)src[k] * scale;
        std::snprintf(name, sizeof(name), stem_fmt, event);
        if (four) write_4col(grid.data(), info_.nx, info_.ny, params_, np, name, binary_);
        if (block) write_block(grid.data(), info_.nx, info_.ny, name, binary_);
      };
      if (sd) {
        std::snprintf(pattern, sizeof(pattern), "data/sn_ecc_eccp_%%d_event_%d.dat", event);
        const double *er = ecc.data() + (size_t)e * 49;
        if (deformed)
          check(smc_write_ecc_deformed(er, ori.data() + (size_t)e * 4, 1, from, to, pattern), "smc_write_ecc_deformed");
        else
          check(smc_write_ecc(er, 1, from, to, pattern), "smc_write_ecc");
        grids(rho.data() + (size_t)e * g, ff, "data/sd_event_%d");
      }
      if (rhob_on) grids(rb.data() + (size_t)e * g, 1.0, "data/rho_binary_event_%d");
      if (ta_on && thick_ok) {
        grids(ta.data() + (size_t)e * g, 1.0, "data/nuclear_thickness_TA_event_%d");
        grids(tb.data() + (size_t)e * g, 1.0, "data/nuclear_thickness_TB_event_%d");
      }
      if (nb_on && thick_ok) {   // net baryon density T_A + T_B
        for (size_t k = 0; k < g; k++) grid[k] = (double)ta[(size_t)e * g + k] + (double)tb[(size_t)e * g + k];
        std::snprintf(name, sizeof(name), "data/rhob_event_%d", event);
        if (four) write_4col(grid.data(), info_.nx, info_.ny, params_, np, name, binary_);
        if (block) write_block(grid.data(), info_.nx, info_.ny, name, binary_);
      }
      if (spect_on) {
        grids(spa.data() + (size_t)e * g, 1.0, "data/spectator_density_A_event_%d");
        grids(spb.data() + (size_t)e * g, 1.0, "data/spectator_density_B_event_%d");
      }
      event++;
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
      std::snprintf(name, sizeof(name), "data/%s_%d", stem[k], order);
      if (four) write_4col(m, info_.nx, info_.ny, params_, 0.0, name, binary_);
      if (block) write_block(m, info_.nx, info_.ny, name, binary_);
    }
  }
}

}  // namespace smc
