// Parity-checker harness around the reference superMC sources.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
// reference's own translation units (src/*.cpp of chunshen1987/superMC, built
// from where they lie by oracle/Makefile.ref) into oracle/_ref/libsmc_ref.so.
// It lets the tests and the fixture generator drive the reference's real code
// on given inputs:
//   * nucleon positions are injected into MCnucl's two Nucleus objects
//     (src/MCnucl.h:25-26), then the reference's getBinaryCollision
//     (src/MCnucl.cpp:217), calculateThickness (:398), setDensity (:626),
//     rotateGrid (:1152) and MakeDensity::dumpEccentricities
//     (src/MakeDensity.cpp:2244) run unchanged;
//   * the native sampler (Nucleus::populate, src/Nucleus.cpp:187) and the
//     whole op-9 event loop (MakeDensity::generateEccTable,
//     src/MakeDensity.cpp:2108) run with a given drand48 seed;
//   * the KLN integrand (KLNModel::func, src/KLNModel.cpp:219) and the
//     BASES-integrated dN/dy (KLNModel::getdNdy, :97) are exposed pointwise;
//   * small numerical helpers (sixPoint2dInterp, Regge96 cross sections,
//     GaussianNucleonsCal::getSigEff, HulthenFunc) are exposed directly.
// No reference source is modified; protected members are reached through
// derived helper classes.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <fstream>
#include <sstream>
#include <unistd.h>
#include <sys/stat.h>

#include "MakeDensity.h"
#include "MCnucl.h"
#include "Nucleus.h"
#include "Particle.h"
#include "KLNModel.h"
#include "KLNfunc.h"
#include "ParameterReader.h"
#include "GaussianNucleonsCal.h"
#include "HulthenFunc.h"
#include "Regge96.h"
#include "arsenal.h"

namespace {

// Reaches the protected members of MCnucl (src/MCnucl.h:24-84).
struct MCAccess : public MCnucl {
  static Nucleus *proj_of(MCnucl *m) { return static_cast<MCAccess *>(m)->proj; }
  static Nucleus *targ_of(MCnucl *m) { return static_cast<MCAccess *>(m)->targ; }
  static std::vector<CollisionPair *> &coll_of(MCnucl *m) {
    return static_cast<MCAccess *>(m)->binaryCollision;
  }
  static void set_table(MCnucl *m, double ***tab, int tmax, double dT) {
    MCAccess *a = static_cast<MCAccess *>(m);
    a->dndyTable = tab;
    a->tmax = tmax;
    a->dT = dT;
  }
  static int maxx(MCnucl *m) { return static_cast<MCAccess *>(m)->Maxx; }
  static int maxy(MCnucl *m) { return static_cast<MCAccess *>(m)->Maxy; }
  static double get_dsq(MCnucl *m) { return static_cast<MCAccess *>(m)->dsq; }
  static double get_width(MCnucl *m) { return static_cast<MCAccess *>(m)->gaussCal->width; }
  static double get_sigma_gg(MCnucl *m) { return static_cast<MCAccess *>(m)->gaussCal->sigma_gg; }
  static double get_siginNN(MCnucl *m) { return static_cast<MCAccess *>(m)->siginNN; }
};

// Reaches MakeDensity::mc (src/MakeDensity.h:17).
struct MDAccess : public MakeDensity {
  static MCnucl *mc_of(MakeDensity *d) { return static_cast<MDAccess *>(d)->mc; }
};

// Exposes the protected KLN integrand (src/KLNModel.h:83).
struct KLNAccess : public KLNModel {
  KLNAccess(double srt, int mode, UnintegPartonDist *f) : KLNModel(srt, mode, f) {}
  double integrand(double *x) { return func(x); }
};

ParameterReader *g_par = 0;
MakeDensity *g_md = 0;
std::string g_workdir;
double ***g_table = 0;
int g_table_n = 0;

void write_quark_table(const std::string &dir) {
  // The reference indexes tables/QuarkPos.txt with (int)(250000*drand48())
  // in every Particle constructor (src/Particle.cpp:38); the real table is
  // not distributed, so an all-zero table (quarks at the nucleon centre)
  // stands in.  It keeps each participant box exactly +-4w.
  std::string tdir = dir + "/tables";
  mkdir(tdir.c_str(), 0755);
  std::string f = tdir + "/QuarkPos.txt";
  FILE *fp = fopen(f.c_str(), "w");
  if (!fp) return;
  for (int i = 0; i < 250001; i++) fputs("0 0 1\n", fp);
  fclose(fp);
}

MCnucl *mc() { return MDAccess::mc_of(g_md); }

void free_table() {
  if (!g_table) return;
  for (int i = 0; i < g_table_n; i++) delete[] g_table[0][i];
  delete[] g_table[0];
  delete[] g_table;
  g_table = 0;
  g_table_n = 0;
}

void push_nucleons(Nucleus *n, const double *xy, int cnt) {
  std::vector<Particle *> &v = n->getNucleons();
  for (int i = 0; i < cnt; i++) v.push_back(new Particle(xy[2 * i], xy[2 * i + 1], 0.0));
  std::sort(v.begin(), v.end(), Nucleus::sortByXLeft);
}

}  // namespace

extern "C" {

// Creates the working directory layout the reference expects (tables/,
// data/, EOS/ link), parses the parameter text (one key=value per line, the
// parameters.dat syntax) and constructs the reference MakeDensity.
int refh_init(const char *workdir, const char *eos_dir, const char *params_text) {
  if (g_md) {
    // the installed dN/dy table belongs to the harness, not to MCnucl
    if (g_table) MCAccess::set_table(mc(), 0, 0, 0.0);
    delete g_md;
    g_md = 0;
  }
  if (g_par) { delete g_par; g_par = 0; }
  free_table();
  g_workdir = workdir;
  mkdir(workdir, 0755);
  write_quark_table(g_workdir);
  mkdir((g_workdir + "/data").c_str(), 0755);
  std::string eos = g_workdir + "/EOS";
  unlink(eos.c_str());
  if (symlink(eos_dir, eos.c_str()) != 0) return -2;
  if (chdir(workdir) != 0) return -1;
  Particle::quark_pos.clear();
  g_par = new ParameterReader;
  std::istringstream in(params_text);
  std::string line;
  while (std::getline(in, line)) g_par->phraseOneLine(line);
  g_md = new MakeDensity(g_par);
  return 0;
}

void refh_srand(long seed) { srand48(seed); srand((unsigned)seed); }

// Injected event: positions (x,y) for projectile and target; the reference's
// own pairing, thickness and density routines run on them.
int refh_inject_event(const double *xyA, int A, const double *xyB, int B, int *npart1,
                      int *npart2, int *ncoll, int do_density) {
  MCnucl *m = mc();
  m->deleteNucleus();
  push_nucleons(MCAccess::proj_of(m), xyA, A);
  push_nucleons(MCAccess::targ_of(m), xyB, B);
  int nc = m->getBinaryCollision();
  *npart1 = m->getNpart1();
  *npart2 = m->getNpart2();
  *ncoll = m->getNcoll();
  if (do_density) {
    m->calculateThickness();
    m->setDensity(0, -1);
  }
  return nc;
}

int refh_grid_dims(int *nx, int *ny) {
  *nx = MCAccess::maxx(mc());
  *ny = MCAccess::maxy(mc());
  return 0;
}

// which: 0 = T_A (projectile), 1 = T_B (target), 2 = rho (rapidity slice 0)
void refh_get_grid(int which, double *out) {
  MCnucl *m = mc();
  int nx = MCAccess::maxx(m), ny = MCAccess::maxy(m);
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double v = 0;
      if (which == 0) v = m->getTA1(i, j);
      else if (which == 1) v = m->getTA2(i, j);
      else v = m->getRho(0, i, j);
      out[(size_t)i * ny + j] = v;
    }
}

// Participant list of one nucleus (0 = projectile) in the reference's
// first-hit order; returns the count.
int refh_participants(int which, double *xy, int maxn) {
  MCnucl *m = mc();
  Nucleus *n = which == 0 ? MCAccess::proj_of(m) : MCAccess::targ_of(m);
  std::vector<Particle *> &p = n->getParticipants();
  int c = (int)p.size();
  for (int i = 0; i < c && i < maxn; i++) {
    xy[2 * i] = p[i]->getX();
    xy[2 * i + 1] = p[i]->getY();
  }
  return c;
}

int refh_nucleons(int which, double *xyz, int maxn) {
  MCnucl *m = mc();
  Nucleus *n = which == 0 ? MCAccess::proj_of(m) : MCAccess::targ_of(m);
  std::vector<Particle *> &p = n->getNucleons();
  int c = (int)p.size();
  for (int i = 0; i < c && i < maxn; i++) {
    xyz[3 * i] = p[i]->getX();
    xyz[3 * i + 1] = p[i]->getY();
    xyz[3 * i + 2] = p[i]->getZ();
  }
  return c;
}

int refh_collisions(double *xy, int maxn) {
  std::vector<CollisionPair *> &c = MCAccess::coll_of(mc());
  int n = (int)c.size();
  for (int i = 0; i < n && i < maxn; i++) {
    xy[2 * i] = c[i]->getX();
    xy[2 * i + 1] = c[i]->getY();
  }
  return n;
}

// Runs MakeDensity::setSd + dumpEccentricities on the current density and
// parses the all-orders line it appends (orders 1..9: Re,Im r^2-weighted,
// Re,Im r^n-weighted, <r^n>; then Npart, Ncoll, integral, b).  out gets 49
// numbers.  The file is written with 8 significant digits.
int refh_eccentricities(int from_order, int to_order, double npart, double ncoll, double b,
                        double *out) {
  MCnucl *m = mc();
  int nx = MCAccess::maxx(m), ny = MCAccess::maxy(m);
  double ***dens = new double **[1];
  dens[0] = new double *[nx];
  for (int i = 0; i < nx; i++) dens[0][i] = new double[ny];
  g_md->setSd(dens, 0);
  remove("data/refh_ecc_10.dat");
  for (int o = 1; o < 10; o++) {
    char fn[64];
    snprintf(fn, sizeof fn, "data/refh_ecc_%d.dat", o);
    remove(fn);
  }
  char base[] = "data/refh_ecc_%d.dat";
  g_md->dumpEccentricities(base, dens, 0, from_order, to_order, npart, ncoll, b);
  for (int i = 0; i < nx; i++) delete[] dens[0][i];
  delete[] dens[0];
  delete[] dens;
  std::ifstream f("data/refh_ecc_10.dat");
  int k = 0;
  double v;
  while (k < 49 && (f >> v)) out[k++] = v;
  return k;
}

// Reference averaged-mode step for one order (src/MakeDensity.cpp:1331-1334):
// rotate the sources to the order-n participant plane about the density's
// centre of mass, then recompute thickness and density.
void refh_rotate_and_resplat(int order) {
  MCnucl *m = mc();
  m->rotateGrid(0, order);
  m->calculateThickness();
  m->setDensity(0, -1);
}

// calculateThickness + setDensity of the current event (after
// refh_sample_event), as the averaged mode does first (src/MakeDensity.cpp:1264,1275).
void refh_density() {
  MCnucl *m = mc();
  m->calculateThickness();
  m->setDensity(0, -1);
}

// Reaction-plane-frame step of the averaged mode (src/MakeDensity.cpp:1291-1293):
// recenter the sources on the density's centre of mass, recompute.
void refh_recenter_and_resplat(int order) {
  MCnucl *m = mc();
  m->recenterGrid(0, order);
  m->calculateThickness();
  m->setDensity(0, -1);
}

// The op-9 event loop of the reference with its native sampler
// (MakeDensity::generateEccTable); results are appended by the reference to
// data/sn_ecc_eccp_*.dat in the working directory.
void refh_generate_ecc_table(int nev) {
  for (int o = 1; o <= 10; o++) {
    char fn[64];
    snprintf(fn, sizeof fn, "data/sn_ecc_eccp_%d.dat", o);
    remove(fn);
  }
  g_md->generateEccTable(nev);
}

// One native-sampler attempt: generateNuclei(b) then getBinaryCollision.
int refh_sample_event(double b, int *npart1, int *npart2, int *ncoll) {
  MCnucl *m = mc();
  m->deleteNucleus();
  m->generateNuclei(b);
  int r = m->getBinaryCollision();
  *npart1 = m->getNpart1();
  *npart2 = m->getNpart2();
  *ncoll = m->getNcoll();
  return r;
}

// Nucleus::populate of one nucleus alone (projectile if which==0).
int refh_populate(int which, double xc, double yc, double *xyz, int maxn) {
  MCnucl *m = mc();
  m->deleteNucleus();
  Nucleus *n = which == 0 ? MCAccess::proj_of(m) : MCAccess::targ_of(m);
  n->populate(xc, yc);
  return refh_nucleons(which, xyz, maxn);
}

// Installs a dN/dy table (row-major tmax x tmax, rapidity slice 0) with
// thickness step dT into MCnucl, as MCnucl::makeTable would have.
void refh_set_kln_table(const double *tab, int tmax, double dT) {
  if (g_table) MCAccess::set_table(mc(), 0, 0, 0.0);
  free_table();
  g_table = new double **[1];
  g_table[0] = new double *[tmax];
  for (int i = 0; i < tmax; i++) {
    g_table[0][i] = new double[tmax];
    for (int j = 0; j < tmax; j++) g_table[0][i][j] = tab[(size_t)i * tmax + j];
  }
  g_table_n = tmax;
  MCAccess::set_table(mc(), g_table, tmax, dT);
}

double refh_sigma_in(double ecm) {
  double sig = hadronxsec::totalXsection(ecm, 0);
  double sigel = hadronxsec::elasticXsection(sig, ecm, 0, 0);
  return sig - sigel;
}

void refh_constants(double *out) {
  MCnucl *m = mc();
  out[0] = MCAccess::get_dsq(m);
  out[1] = MCAccess::get_width(m);
  out[2] = MCAccess::get_sigma_gg(m);
  out[3] = MCAccess::get_siginNN(m);
}

double refh_six_point(double x, double y, double v00, double v01, double v02, double v10,
                      double v11, double v20) {
  return sixPoint2dInterp(x, y, v00, v01, v02, v10, v11, v20);
}

double refh_hulthen_cdf(double r) { return HulthenFunc::CDF(r); }
double refh_hulthen_inv(double u) {
  HulthenFunc h;
  return h.invCDF(u);
}

// KLN: integrand at the unit-cube point x[3] (pt, kt, phi fractions), and
// the BASES integral, both for thicknesses (ta, tb) at rapidity y.
static KLNAccess *g_kln = 0;
static KLNfunc *g_klnf = 0;
void refh_kln_setup(double ecm, double lambda) {
  if (g_kln) { delete g_kln; delete g_klnf; }
  g_klnf = new KLNfunc();
  g_kln = new KLNAccess(ecm, KLN, g_klnf);
  g_kln->setLambdaSaturation(lambda);
  g_kln->setNormalization(1.0);
}
double refh_kln_integrand(double y, double ta, double tb, double x0, double x1, double x2) {
  // getdNdy stores (Npart1, Npart2, rapidity, partonPt, PT_order) before
  // integrating; a zero-sample call is not available, so set them through a
  // cheap fixed-pt call first and then evaluate func directly.
  (void)y;
  double x[3] = {x0, x1, x2};
  return g_kln->integrand(x);
}
void refh_kln_prepare(double y, double ta, double tb) {
  // Sets the integrand state exactly as getdNdy does (src/KLNModel.cpp:99-104)
  // by running the pt-integrated path once with the same arguments.
  g_kln->getdNdy(y, ta, tb, -1.0, 1);
}
double refh_kln_dndy(double y, double ta, double tb) { return g_kln->getdNdy(y, ta, tb, -1.0, 1); }
// dN/dy d^2p_T at fixed p_T (the adaptive-Simpson path, src/KLNModel.cpp:115-119)
double refh_kln_dndy_pt(double y, double ta, double tb, double pt) { return g_kln->getdNdy(y, ta, tb, pt, 1); }
double refh_kln_norm() { return KLNModel::Norm; }

}  // extern "C"
