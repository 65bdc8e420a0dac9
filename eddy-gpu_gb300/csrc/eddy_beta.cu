// eddy_beta.cu -- the beta fit of each set's JS values and its pDDN, on the
// device, for every set of a run in one launch (main.cu:1488-1502,
// routines.cu:494-508).
//
// The JS values of a run stay on the device (the JS kernel writes each one
// into the run's array as well), so the fit needs no copy in.  One thread
// per set keeps the reference's sequential summation order: the moments,
// alpha and beta are rounded exactly as the host loop rounds them.  The
// reference's boost::math::ibetac is replaced by the continued fraction of
// the regularised incomplete beta function (DLMF 8.17.22) evaluated with
// the modified Lentz method (Lentz 1976; Thompson & Barnett 1986), with
// CUDA's own log, log1p, lgamma and exp.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "eddy_kernels.h"

namespace eddy {
namespace {

// 1 / (1 + d1 / (1 + d2 / (1 + ...))) of I_x(a, b) = x^a (1-x)^b / (a B(a, b))
// * (that fraction), with
//   d_{2m+1} = -(a+m)(a+b+m) x / ((a+2m)(a+2m+1)),
//   d_{2m}   =  m (b-m) x / ((a+2m-1)(a+2m)).
__device__ double beta_cf(double a, double b, double x) {
  const double tiny = 1e-300;
  double f = 1.0, C = 1.0, D = 0.0;
  for (int j = 1; j <= 400000; j++) {
    const int m = j / 2;
    const double dj = (j & 1) ? -((a + m) * (a + b + m) * x) / ((a + 2.0 * m) * (a + 2.0 * m + 1.0))
                              : (m * (b - m) * x) / ((a + 2.0 * m - 1.0) * (a + 2.0 * m));
    D = 1.0 + dj * D;
    if (fabs(D) < tiny) D = tiny;
    D = 1.0 / D;
    C = 1.0 + dj / C;
    if (fabs(C) < tiny) C = tiny;
    const double delta = C * D;
    f *= delta;
    if (fabs(delta - 1.0) < 1e-15) break;
  }
  return 1.0 / f;
}

__device__ double ibeta_lower(double a, double b, double x) {
  const double lfront = a * log(x) + b * log1p(-x) - (lgamma(a) + lgamma(b) - lgamma(a + b));
  return exp(lfront) / a * beta_cf(a, b, x);
}

// 1 - I_x(a, b); the fraction converges fast for x below the mean
// (a+1)/(a+b+2), so above it the symmetric form I_{1-x}(b, a) is summed.
__device__ double ibetac(double a, double b, double x) {
  if (x == 0) return 1.0;
  if (x == 1) return 0.0;
  if (x < (a + 1.0) / (a + b + 2.0)) return 1.0 - ibeta_lower(a, b, x);
  return ibeta_lower(b, a, 1.0 - x);
}

// out[4 i ..]: alpha, beta, pDDN, 1.0 (fit valid) or 0.0, for the R[i]
// values js_all[off[i] ..].  The moments use explicit round-to-nearest
// operations (no contraction) in the host loop's order.
__global__ void k_beta_fit(const double *js_all, const long long *off, const int *R, int nsets,
                           double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsets) return;
  const double *js = js_all + off[i];
  const int r = R[i];
  double sum = 0.0;
  for (int k = 0; k < r; k++) sum = __dadd_rn(sum, js[k]);
  const double mu = __ddiv_rn(sum, (double)r);
  double v = 0.0;
  for (int k = 0; k < r; k++) {
    const double d = __dsub_rn(js[k], mu);
    v = __dadd_rn(v, __dmul_rn(d, d));
  }
  const double var = __ddiv_rn(v, (double)r);
  const double t = __dsub_rn(__ddiv_rn(__dsub_rn(1.0, mu), var), __ddiv_rn(1.0, mu));
  const double alpha = __dmul_rn(t, __dmul_rn(mu, mu));
  const double beta = __dmul_rn(alpha, __dsub_rn(__ddiv_rn(1.0, mu), 1.0));
  const double j0 = js[0];
  const bool ok = alpha > 0 && beta > 0 && isfinite(alpha) && isfinite(beta) && j0 >= 0 && j0 <= 1;
  out[4 * (size_t)i + 0] = alpha;
  out[4 * (size_t)i + 1] = beta;
  out[4 * (size_t)i + 2] = ok ? ibetac(alpha, beta, j0) : __longlong_as_double(0x7ff8000000000000ll);
  out[4 * (size_t)i + 3] = ok ? 1.0 : 0.0;
}

}  // namespace

cudaError_t launch_beta_fit(const double *js_all, const long long *off, const int *R, int nsets,
                            double *out, cudaStream_t st) {
  if (nsets <= 0) return cudaSuccess;
  k_beta_fit<<<(nsets + 63) / 64, 64, 0, st>>>(js_all, off, R, nsets, out);
  return cudaGetLastError();
}

}  // namespace eddy
