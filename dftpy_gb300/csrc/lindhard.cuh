// Inverse Lindhard function (FP64, device).
//
//   L(eta) = 1 / F(eta) - 3 mu eta^2 - lbda,
//   F(eta) = 1/2 + (1 - eta^2) / (4 eta) ln|(1 + eta) / (1 - eta)|,
// with the reference's large-eta series for eta > 3.65 and its limits at
// eta = 0 and eta = 1 (kedf/kernel.py:14-136).
#pragma once
#include <math.h>

namespace gblind {

static __constant__ double c_lind_large[15] = {
    -0.13714285714285712,    -6.39999999999999875e-2, -3.77825602968460128e-2, -2.51824061652633074e-2,
    -1.80879839616166146e-2, -1.36715733124818332e-2, -1.07236045520990083e-2, -8.65192783339199453e-3,
    -7.1372762502456763e-3,  -5.9945117538835746e-3,  -5.10997527675418131e-3, -4.41060829979912465e-3,
    -3.84763737842981233e-3, -3.38745061493813488e-3, -3.00624946457977689e-3};

__device__ __forceinline__ double lindhard_inv(double eta, double lbda, double mu) {
  if (eta > 3.65) {
    const double inv = 1.0 / (eta * eta);
    double s = c_lind_large[14];
    for (int i = 13; i >= 0; --i) s = c_lind_large[i] + inv * s;
    return 3.0 * (1.0 - mu) * eta * eta - lbda - 0.6 + inv * s;
  }
  if (fabs(eta - 1.0) < 1e-10) return 2.0 - lbda - 3.0 * mu + 20.0 * (eta - 1.0);
  if (eta < 1e-10) return 1.0 - lbda + eta * eta * (1.0 / 3.0 - 3.0 * mu);
  return 1.0 / (0.5 + 0.25 * (1.0 - eta * eta) * log((1.0 + eta) / fabs(1.0 - eta)) / eta) -
         3.0 * mu * eta * eta - lbda;
}

}  // namespace gblind
