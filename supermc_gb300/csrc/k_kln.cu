// MC-KLN dN/dy lookup table (MCnucl::makeTable, src/MCnucl.cpp:911-960).
//
// The reference integrates KLNModel::func (src/KLNModel.cpp:219-277) over
// (p_T, k_T, phi) with the BASES Monte-Carlo integrator at every table node
// (T_A, T_B) = (i dT, j dT).  Here the same integrand is integrated by a
// deterministic tensor-product Gauss-Legendre rule on the unit cube, one CTA
// per node, in FP64 throughout (the table then equals the FP64 oracle's to
// ~1e-14 relative; the per-cell lookup reads an FP32 copy).  The saturation
// scales Q_s^2(x(p_T)), the wave-function prefactors fac (1-x)^4 / alpha_s(Q_s^2)
// (KLNfunc::getFunc, KLNModel::waveFunction, :381-399) and the Jacobian
// depend only on (p_T, k_T) and are staged in shared memory per p_T node.
// The phi rule is symmetric (nodes x and 1-x carry the same weight and the
// same cos(2 pi x)), so each pair is evaluated once with twice the weight.
// Per evaluation: one log (the running coupling at max(k1^2, k2^2, m_T^2),
// KLNModel.h:91-96) and one division (the saturated wave functions and the
// coupling folded into one quotient).
#include "smc_kernels.h"

namespace smc {

constexpr int kKT = 256;
constexpr int kMaxNodes = 256;

__global__ void __launch_bounds__(kKT) k_kln_table(KlnDev K, int tmax, double dT, double *table64,
                                                   float *table32) {
  __shared__ double s_qa[kMaxNodes], s_qb[kMaxNodes], s_fab[kMaxNodes], s_pt[kMaxNodes], s_pw[kMaxNodes];
  __shared__ double s_cos[kMaxNodes / 2 + 1], s_fw[kMaxNodes / 2 + 1], s_kx[kMaxNodes], s_kw[kMaxNodes];
  __shared__ double s_red[kKT / 32];
  const int node = blockIdx.x;
  const int i = node / tmax, j = node % tmax;
  const int tid = threadIdx.x;
  if (i == 0 || j == 0) {   // MCnucl.cpp:937-944
    if (tid == 0) { table64[node] = 0.0; table32[node] = 0.f; }
    return;
  }
  const double ta = dT * i, tb = dT * j;
  const double inv_l2 = 1.0 / K.lambda_qcd2, inv_amax = 1.0 / K.alpha_max;
  // alpha_s(q2) = min(alpha_max, 1 / (beta0 ln(q2 / Lambda^2))), alpha_max at q2 <= Lambda^2
  auto alpha_s = [&](double q2) {
    if (q2 <= K.lambda_qcd2) return K.alpha_max;
    const double v = 1.0 / (K.beta0 * log(q2 * inv_l2));
    return K.alpha_max < v ? K.alpha_max : v;
  };
  for (int p = tid; p < K.npt; p += kKT) {
    const double pt = K.ptmin + K.xp[p] * (K.ptmax - K.ptmin);
    const double x1 = pt / K.ecm * exp(K.y), x2 = pt / K.ecm / exp(K.y);
    const bool ok = !(x1 > 1.0 || x2 > 1.0);
    const double qa = ta * 2. / 1.53 * pow(0.01 / x1, K.lambda);   // KLNModel::SaturationScale
    const double qb = tb * 2. / 1.53 * pow(0.01 / x2, K.lambda);
    const double fa = K.fac * pow(1.0 - x1, 4.) / alpha_s(qa);
    const double fb = K.fac * pow(1.0 - x2, 4.) / alpha_s(qb);
    s_qa[p] = qa;
    s_qb[p] = qb;
    s_fab[p] = ok ? fa * fb : 0.0;
    s_pt[p] = pt;
    s_pw[p] = K.wp[p];
  }
  const int nh = K.nphi / 2, nf = nh + (K.nphi & 1);
  for (int f = tid; f < nf; f += kKT) {
    s_cos[f] = K.cf[f];
    s_fw[f] = f < nh ? 2.0 * K.wf[f] : K.wf[f];
  }
  for (int k = tid; k < K.nkt; k += kKT) { s_kx[k] = K.xk[k]; s_kw[k] = K.wk[k]; }
  __syncthreads();
  const double dpt = K.ptmax - K.ptmin;
  const double pi2 = M_PI * M_PI;
  double acc = 0.0;
  for (int pk = tid; pk < K.npt * K.nkt; pk += kKT) {
    const int p = pk / K.nkt, k = pk - p * K.nkt;
    const double fab = s_fab[p];
    if (fab == 0.0) continue;
    const double pt = s_pt[p], kt = pt * s_kx[k];
    const double qa = s_qa[p], qb = s_qb[p];
    const double pt2 = pt * pt, base = 0.25 * (pt2 + kt * kt), cross = 0.5 * kt * pt;
    double sum = 0.0;
    for (int f = 0; f < nf; f++) {
      const double c = s_cos[f];
      const double k1 = base + cross * c, k2 = base - cross * c;
      // phi_A phi_B alpha_s(scale) = fab [qa/k1] [qb/k2] / D, the saturated
      // factors only beyond Q_s^2, and D = 1/alpha_s(scale)
      double num = fab, den = 1.0;
      if (k1 > qa) { num *= qa; den *= k1; }
      if (k2 > qb) { num *= qb; den *= k2; }
      const double scale = fmax(fmax(k1, k2), pt2);
      double d = inv_amax;
      if (scale > K.lambda_qcd2) d = fmax(d, K.beta0 * log(scale * inv_l2));
      sum += s_fw[f] * (num / (den * d));
    }
    // 2 pi (Ptmax-Ptmin) pt / mt^2 * 2 pi kt ktmax / 4 = pi^2 (Ptmax-Ptmin) kt   (mt = ktmax = pt)
    acc += sum * (pi2 * dpt * kt) * s_kw[k] * s_pw[p];
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((tid & 31) == 0) s_red[tid >> 5] = acc;
  __syncthreads();
  if (tid == 0) {
    double s = 0;
    for (int w = 0; w < kKT / 32; w++) s += s_red[w];
    const double v = K.prefactor * s;   // 1.0 * g2hfac * Norm * I * 9/32 (KLNModel.cpp:109)
    table64[node] = v;
    table32[node] = (float)v;
  }
}

cudaError_t launch_kln_table(const KlnDev &K, int tmax, double dT, double *table64, float *table32,
                             cudaStream_t st) {
  if (K.npt > kMaxNodes || K.nkt > kMaxNodes || K.nphi > kMaxNodes) return cudaErrorInvalidValue;
  k_kln_table<<<tmax * tmax, kKT, 0, st>>>(K, tmax, dT, table64, table32);
  return cudaGetLastError();
}

// p_T-differential dN/dy d^2p_T table (MCnucl::makeTable(ptmin, dpt, iPtmax),
// src/MCnucl.cpp:967-1025): at every node (T_A, T_B) = (i dT, j dT) and
// p_T bin p (p_T = ptmin + p dpt), KLNModel::getdNdy at fixed p_T
// (src/KLNModel.cpp:96-124): prefactor times the (k_T, phi) integral of
// KLNModel::func_simpson (:281-322) over k_T in [0, p_T], phi in [0, 2 pi],
// which the reference takes by adaptive Simpson (relative precision 1e-4)
// and which is taken here by the tensor-product Gauss-Legendre rule of the
// p_T-integrated table (k_T and phi nodes), in FP64.  One CTA per node; the
// warps take the p_T bins in turn, the lanes the k_T nodes, and each bin's
// sum is reduced in a fixed order.  Layout [tmax][tmax][nbins].
__global__ void __launch_bounds__(kKT) k_kln_pt_table(KlnDev K, int tmax, double dT, double ptmin, double dpt,
                                                      int nbins, double *table64, float *table32) {
  __shared__ double s_cos[kMaxNodes / 2 + 1], s_fw[kMaxNodes / 2 + 1], s_kx[kMaxNodes], s_kw[kMaxNodes];
  const int node = blockIdx.x;
  const int i = node / tmax, j = node % tmax;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  double *out64 = table64 + (size_t)node * nbins;
  float *out32 = table32 + (size_t)node * nbins;
  if (i == 0 || j == 0) {   // MCnucl.cpp:1006-1012
    for (int p = tid; p < nbins; p += kKT) { out64[p] = 0.0; out32[p] = 0.f; }
    return;
  }
  const double ta = dT * i, tb = dT * j;
  const double inv_l2 = 1.0 / K.lambda_qcd2, inv_amax = 1.0 / K.alpha_max;
  auto alpha_s = [&](double q2) {
    if (q2 <= K.lambda_qcd2) return K.alpha_max;
    const double v = 1.0 / (K.beta0 * log(q2 * inv_l2));
    return K.alpha_max < v ? K.alpha_max : v;
  };
  const int nh = K.nphi / 2, nf = nh + (K.nphi & 1);
  for (int f = tid; f < nf; f += kKT) {
    s_cos[f] = K.cf[f];
    s_fw[f] = f < nh ? 2.0 * K.wf[f] : K.wf[f];
  }
  for (int k = tid; k < K.nkt; k += kKT) { s_kx[k] = K.xk[k]; s_kw[k] = K.wk[k]; }
  __syncthreads();
  for (int p = wid; p < nbins; p += kKT / 32) {
    const double pt = ptmin + p * dpt;
    const double x1 = pt / K.ecm * exp(K.y), x2 = pt / K.ecm / exp(K.y);
    double acc = 0.0;
    if (!(x1 > 1.0 || x2 > 1.0) && pt > 0.0) {
      const double qa = ta * 2. / 1.53 * pow(0.01 / x1, K.lambda);   // KLNModel::SaturationScale
      const double qb = tb * 2. / 1.53 * pow(0.01 / x2, K.lambda);
      const double fab = K.fac * pow(1.0 - x1, 4.) / alpha_s(qa) * (K.fac * pow(1.0 - x2, 4.) / alpha_s(qb));
      const double pt2 = pt * pt;
      for (int k = lane; k < K.nkt; k += 32) {
        const double kt = pt * s_kx[k];
        const double base = 0.25 * (pt2 + kt * kt), cross = 0.5 * kt * pt;
        double sum = 0.0;
        for (int f = 0; f < nf; f++) {
          const double c = s_cos[f];
          const double k1 = base + cross * c, k2 = base - cross * c;
          double num = fab, den = 1.0;
          if (k1 > qa) { num *= qa; den *= k1; }
          if (k2 > qb) { num *= qb; den *= k2; }
          const double scale = fmax(fmax(k1, k2), pt2);
          double d = inv_amax;
          if (scale > K.lambda_qcd2) d = fmax(d, K.beta0 * log(scale * inv_l2));
          sum += s_fw[f] * (num / (den * d));
        }
        // (pt dk)(2 pi dphi) kt / (4 pt^2) = pi kt / (2 pt) per unit of the [0,1] rules
        acc += sum * (M_PI * kt / (2.0 * pt)) * s_kw[k];
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const double v = K.prefactor * acc;
      out64[p] = v;
      out32[p] = (float)v;
    }
  }
}

cudaError_t launch_kln_pt_table(const KlnDev &K, int tmax, double dT, double ptmin, double dpt, int nbins,
                                double *table64, float *table32, cudaStream_t st) {
  if (K.nkt > kMaxNodes || K.nphi > kMaxNodes || nbins < 1) return cudaErrorInvalidValue;
  k_kln_pt_table<<<tmax * tmax, kKT, 0, st>>>(K, tmax, dT, ptmin, dpt, nbins, table64, table32);
  return cudaGetLastError();
}

}  // namespace smc
