// MC-KLN dN/dy lookup table (MCnucl::makeTable, src/MCnucl.cpp:911-960).
//
// The reference integrates KLNModel::func (src/KLNModel.cpp:219-277) over
// (p_T, k_T, phi) with the BASES Monte-Carlo integrator at every table node
// (T_A, T_B) = (i dT, j dT).  Here the same integrand is integrated by a
// deterministic tensor-product Gauss-Legendre rule on the unit cube, one CTA
// per node.  The saturation scales Q_s^2(x(p_T)), their running couplings and
// the (1-x)^4 factors depend only on (p_T node, thickness) and are staged in
// shared memory; cos(phi) per phi node likewise.
#include "smc_kernels.h"

namespace smc {

constexpr int kKT = 256;
constexpr int kMaxNodes = 256;

__device__ __forceinline__ float alpha_s(float q2, float l2, float amax, float beta0) {
  if (q2 <= l2) return amax;
  return fminf(amax, 1.0f / (beta0 * logf(q2 / l2)));
}

__global__ void __launch_bounds__(kKT) k_kln_table(KlnDev K, int tmax, double dT, double *table64,
                                                   float *table32) {
  __shared__ float s_qa[kMaxNodes], s_qb[kMaxNodes], s_fa[kMaxNodes], s_fb[kMaxNodes], s_pt[kMaxNodes];
  __shared__ float s_pw[kMaxNodes], s_cos[kMaxNodes], s_fw[kMaxNodes], s_kx[kMaxNodes], s_kw[kMaxNodes];
  __shared__ double s_red[kKT / 32];
  const int node = blockIdx.x;
  const int i = node / tmax, j = node % tmax;
  const int tid = threadIdx.x;
  if (i == 0 || j == 0) {   // MCnucl.cpp:937-944
    if (tid == 0) { table64[node] = 0.0; table32[node] = 0.f; }
    return;
  }
  const double ta = dT * i, tb = dT * j;
  const float l2 = (float)K.lambda_qcd2, amax = (float)K.alpha_max, beta0 = (float)K.beta0;
  for (int p = tid; p < K.npt; p += kKT) {
    double pt = K.ptmin + K.xp[p] * (K.ptmax - K.ptmin);
    double x1 = pt / K.ecm * exp(K.y), x2 = pt / K.ecm / exp(K.y);
    bool ok = !(x1 > 1.0 || x2 > 1.0);
    double qa = ta * 2. / 1.53 * pow(0.01 / x1, K.lambda);   // KLNModel::SaturationScale
    double qb = tb * 2. / 1.53 * pow(0.01 / x2, K.lambda);
    // KLNfunc::getFunc / waveFunction prefactors: fac / alpha_s(Qs^2) (1-x)^4
    float fa = (float)(K.fac * pow(1.0 - x1, 4.)) / alpha_s((float)qa, l2, amax, beta0);
    float fb = (float)(K.fac * pow(1.0 - x2, 4.)) / alpha_s((float)qb, l2, amax, beta0);
    s_qa[p] = (float)qa; s_qb[p] = (float)qb;
    s_fa[p] = ok ? fa : 0.f; s_fb[p] = fb;
    s_pt[p] = (float)pt;
    s_pw[p] = (float)K.wp[p];
  }
  for (int f = tid; f < K.nphi; f += kKT) {
    s_cos[f] = (float)cos(2 * M_PI * K.xf[f]);
    s_fw[f] = (float)K.wf[f];
  }
  for (int k = tid; k < K.nkt; k += kKT) { s_kx[k] = (float)K.xk[k]; s_kw[k] = (float)K.wk[k]; }
  __syncthreads();
  const float dpt = (float)(K.ptmax - K.ptmin);
  const float two_pi = 6.28318530717958647692f;
  double acc = 0.0;
  for (int pk = tid; pk < K.npt * K.nkt; pk += kKT) {
    const int p = pk / K.nkt, k = pk % K.nkt;
    const float pt = s_pt[p], kt = pt * s_kx[k];
    const float qa = s_qa[p], qb = s_qb[p], fa = s_fa[p], fb = s_fb[p];
    const float pt2 = pt * pt, kt2 = kt * kt, base = 0.25f * (pt2 + kt2), cross = 0.5f * kt * pt;
    float sum = 0.f;
    for (int f = 0; f < K.nphi; f++) {
      const float c = s_cos[f];
      const float k1 = base + cross * c, k2 = base - cross * c;
      const float pa = k1 <= qa ? fa : fa * qa / k1;
      const float pb = k2 <= qb ? fb : fb * qb / k2;
      const float scale = fmaxf(fmaxf(k1, k2), pt2);
      sum += s_fw[f] * (alpha_s(scale, l2, amax, beta0) * pa * pb);
    }
    // 2 pi (Ptmax-Ptmin) pt / mt^2 * 2 pi kt ktmax / 4   (mt = pt)
    const float jac = two_pi * dpt * pt / pt2 * two_pi * kt * pt * 0.25f;
    acc += (double)(sum * jac) * (double)s_kw[k] * (double)s_pw[p];
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((tid & 31) == 0) s_red[tid >> 5] = acc;
  __syncthreads();
  if (tid == 0) {
    double s = 0;
    for (int w = 0; w < kKT / 32; w++) s += s_red[w];
    double v = K.prefactor * s;   // 1.0 * g2hfac * Norm * I * 9/32 (KLNModel.cpp:109)
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

}  // namespace smc
