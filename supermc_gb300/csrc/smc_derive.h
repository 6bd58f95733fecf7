// Host-side derivation of the device constants from the configuration,
// shared by the context (smc_capi.cu) and the no-allocation entry point
// (smc_noalloc.cu): sigma_in, the nucleon width and sigma_gg, the nuclei,
// the grid and the model switches (MCnucl::MCnucl, src/MCnucl.cpp:22-154).
#pragma once
#include <algorithm>
#include <cmath>

#include "../../include/supermc.h"
#include "smc_device.cuh"

namespace smc_host {

// sigma_in = sigma_tot - sigma_el for pp from the PDG-96 Regge fits
// (hadronxsec::totalXsection / elasticXsection, src/Regge96.cpp:27-50).
inline double sigma_inelastic(double ecm) {
  double s = ecm * ecm;
  double sig = 22.0 * std::pow(s, 0.079) + 56.1 * std::pow(s, -0.46);
  double bel = 2.0 * 2.3 + 2.0 * 2.3 + 4.0 * std::pow(s, 0.0808) - 4.2;
  return sig - 0.0511 * sig * sig / bel;
}

// 38-point Gauss-Legendre abscissae/weights on [0,1] from the published
// table the reference uses (Nucleus::Gauss38, src/Nucleus.cpp:697-751).
inline void gauss38_unit(double *xn, double *wn) {
  static const double xp[19] = {
      4.078514790458e-2, 1.220840253379e-1, 2.025704538921e-1, 2.817088097902e-1, 3.589724404794e-1,
      4.338471694324e-1, 5.058347179279e-1, 5.744560210478e-1, 6.392544158297e-1, 6.997986803792e-1,
      7.556859037540e-1, 8.065441676053e-1, 8.520350219324e-1, 8.918557390046e-1, 9.257413320486e-1,
      9.534663309335e-1, 9.748463285902e-1, 9.897394542664e-1, 9.980499305357e-1};
  static const double wp[19] = {
      8.152502928039e-2, 8.098249377060e-2, 7.990103324353e-2, 7.828784465821e-2, 7.615366354845e-2,
      7.351269258474e-2, 7.038250706690e-2, 6.678393797914e-2, 6.274093339213e-2, 5.828039914700e-2,
      5.343201991033e-2, 4.822806186076e-2, 4.270315850467e-2, 3.689408159400e-2, 3.083950054518e-2,
      2.457973973823e-2, 1.815657770961e-2, 1.161344471647e-2, 5.002880749632e-3};
  for (int k = 0; k < 19; k++) {
    xn[19 + k] = (1.0 * xp[k]) / 2.0 + 0.5;
    wn[19 + k] = (1.0 * wp[k]) / 2.0;
    xn[18 - k] = (1.0 * -xp[k]) / 2.0 + 0.5;
    wn[18 - k] = (1.0 * wp[k]) / 2.0;
  }
}

// sigma_gg from sigma_in = int d^2b [1 - exp(-sigma_gg T_pp(b))] by Newton
// iteration (GaussianNucleonsCal::getSigEff, src/GaussianNucleonsCal.cpp:130-163).
inline double sigma_gg_from(double siginNN, double width) {
  double xg[38], wg[38];
  gauss38_unit(xg, wg);
  double sigin = siginNN * 0.1, Bmax = 5.0 * width, sigeff = 10.0, prev;
  int guard = 0;
  do {
    prev = sigeff;
    double sum = 0.0, dN = 0.0;
    for (int ib = 0; ib < 38; ib++) {
      double b = xg[ib] * Bmax, db = wg[ib] * Bmax;
      double Tpp = std::exp(-b * b / (4. * width * width)) / (M_PI * (4. * width * width));
      sum += 2 * M_PI * b * db * (1.0 - std::exp(-sigeff * Tpp));
      dN += 2 * M_PI * b * db * Tpp * std::exp(-sigeff * Tpp);
    }
    sigeff -= (sum - sigin) / dN;
  } while (std::fabs(sigeff - prev) > 1e-4 && ++guard < 1000);
  return sigeff;
}

// Nucleus::Nucleus radius/diffuseness/deformation table (src/Nucleus.cpp:58-148)
inline smc::NucleusDev make_nucleus(int A, int deformed, double R_ov, double a_ov, double dmin_ov) {
  smc::NucleusDev n{};
  n.A = A;
  n.deformed = deformed;
  double Ad = A;
  double rad = 1.12 * std::pow(Ad, 0.333333) - 0.86 / std::pow(Ad, 0.333333), dr = 0.54;
  if (A == 197) { rad = 6.42; dr = 0.45; }
  else if (A == 63) { rad = 4.28; dr = 0.5; }
  else if (A == 238) { rad = 6.86; dr = 0.44; }
  else if (A == 208) { rad = 6.67; dr = 0.44; }
  else if (A == 129) { rad = 5.36; dr = 0.590; }
  if (R_ov > 0) rad = R_ov;
  if (a_ov > 0) dr = a_ov;
  n.R = rad;
  n.a = dr;
  n.d_min = dmin_ov > 0 ? dmin_ov : 0.9;
  if (deformed) {
    if (A == 197) { n.beta2 = -0.13; n.beta4 = -0.03; }
    else if (A == 63) { n.beta2 = 0.162; n.beta4 = 0.006; }
    else if (A == 129) { n.beta2 = 0.162; n.beta4 = -0.003; }
    else if (A == 238) { n.beta2 = 0.28; n.beta4 = 0.093; }
  }
  n.rmax_cut = rad + 2.5;
  n.rw_max = 1.0 / (1.0 + std::exp(-rad / dr));
  return n;
}

// The device constants both entry points derive the same way: grid, nucleon
// width and cross sections, the model switches, the Gamma multiplicity
// weights (cc_fluctuation_model 6, src/MCnucl.cpp:1271-1301), the nuclei,
// the eccentricity orders and the widest splat window.  Returns sigma_in.
inline double derive_common(const smc_params &p, smc::DevParams &P) {
  const double sigin = p.sigin_override > 0 ? p.sigin_override : sigma_inelastic(p.ecm);
  double width = 0;
  if (p.shape_of_nucleons == 1) width = std::sqrt(0.1 * sigin / M_PI) / 2.0;
  else if (p.shape_of_nucleons == 2) width = std::sqrt(0.1 * sigin / M_PI) / std::sqrt(8.0);
  else width = p.gauss_nucl_width;
  P.nx = (int)((p.maxx - (-p.maxx)) / p.dx + 0.1) + 1;   // MCnucl.cpp:39-40
  P.ny = (int)((p.maxy - (-p.maxy)) / p.dy + 0.1) + 1;
  P.xmin = -p.maxx; P.ymin = -p.maxy; P.dx = p.dx; P.dy = p.dy;
  P.inv_dx = 1.0 / p.dx; P.inv_dy = 1.0 / p.dy;
  P.width = width; P.w2 = width * width; P.quark_width = p.quark_width;
  P.peak = 1 / (2 * M_PI * width * width);
  P.dsq = 0.1 * sigin / M_PI / 1;                       // MCnucl.cpp:120 (overSample = 1)
  P.sigin = sigin;
  P.sigma_gg = sigma_gg_from(sigin, width);
  P.alpha = p.alpha; P.final_factor = p.final_factor;
  if (p.cc_fluctuation_model == 6) {
    const double eps = 1e-8, th = p.cc_fluctuation_gamma_theta;
    P.fluct = 1;
    P.fluct_k_part = (1 - p.alpha + eps) / 2. * (1. / th);
    P.fluct_th_part = 2. / (1 - p.alpha + eps) * th;
    P.fluct_k_coll = (p.alpha + eps) * (1. / th);
    P.fluct_th_coll = 1. / (p.alpha + eps) * th;
  }
  P.which_mc_model = p.which_mc_model; P.sub_model = p.sub_model;
  P.shape_of_nucleons = p.shape_of_nucleons; P.shape_of_entropy = p.shape_of_entropy;
  P.collision_criterion = p.collision_criterion;
  P.npmin = p.npmin; P.npmax = p.npmax; P.bmin = p.bmin; P.bmax = p.bmax;
  P.nuc[0] = make_nucleus(p.Aproj, p.proj_deformed, p.proj_R, p.proj_a, p.proj_d_min);
  P.nuc[1] = make_nucleus(p.Atarg, p.targ_deformed, p.targ_R, p.targ_a, p.targ_d_min);
  P.seed = p.seed;
  P.ecc_from = p.ecc_from_order; P.ecc_to = p.ecc_to_order;
  const double d_max = p.shape_of_nucleons == 1 ? 2. * std::sqrt(P.dsq) : 5. * width;
  const double span = std::max(2 * d_max, 8 * std::max(width, p.quark_width));
  P.splat_mw = (int)(span / std::min(p.dx, p.dy)) + 3;
  return sigin;
}

}  // namespace smc_host
