// Stencil kernels, exact build: compiled with -fmad=false and IEEE division so each
// multiply, add and divide is rounded separately, in the reference's order. Used by
// the bit-for-bit parity tests and selectable at run time.
#define PGB_NS exact
#define PGB_EXACT_ARITH 1

#include "stencil.cuh"

namespace pgb {
namespace exact {

__device__ __forceinline__ double recip(double x) { return 1.0 / x; }

// WENO5-Z with MC blending, benchmarks/burgers/recon.hpp:42-99 (same expression order).
__device__ __forceinline__ void weno5z(double q0, double q1, double q2, double q3, double q4, double &ql,
                                       double &qr) {
  constexpr double c00 = 1.0 / 3.0, c01 = -7.0 / 6.0, c02 = 11.0 / 6.0;
  constexpr double c10 = -1.0 / 6.0, c11 = 5.0 / 6.0, c12 = 1.0 / 3.0;
  constexpr double c20 = 1.0 / 3.0, c21 = 5.0 / 6.0, c22 = -1.0 / 6.0;
  constexpr double g0 = 0.1, g1 = 0.6, g2 = 0.3;
  constexpr double eps = kWenoEps;
  constexpr double tt = 13.0 / 3.0;
  double a = q0 - 2 * q1 + q2;
  double b = q0 - 4.0 * q1 + 3.0 * q2;
  double be0 = tt * a * a + b * b + eps;
  a = q1 - 2.0 * q2 + q3;
  b = q3 - q1;
  double be1 = tt * a * a + b * b + eps;
  a = q2 - 2.0 * q3 + q4;
  b = q4 - 4.0 * q3 + 3.0 * q2;
  double be2 = tt * a * a + b * b + eps;
  const double tau5 = fabs(be2 - be0);
  be0 = (be0 + tau5) / be0;
  be1 = (be1 + tau5) / be1;
  be2 = (be2 + tau5) / be2;
  double w0 = g0 * be0 + eps;
  double w1 = g1 * be1 + eps;
  double w2 = g2 * be2 + eps;
  double ws = 1.0 / (w0 + w1 + w2);
  ql = w0 * (c00 * q0 + c01 * q1 + c02 * q2);
  ql += w1 * (c10 * q1 + c11 * q2 + c12 * q3);
  ql += w2 * (c20 * q2 + c21 * q3 + c22 * q4);
  ql *= ws;
  const double al = 3.0 * ws * w0 * w1 * w2 / (g2 * w0 * w1 + g1 * w0 * w2 + g0 * w1 * w2) + eps;
  w0 = g0 * be2 + eps;
  w1 = g1 * be1 + eps;
  w2 = g2 * be0 + eps;
  ws = 1.0 / (w0 + w1 + w2);
  qr = w0 * (c00 * q4 + c01 * q3 + c02 * q2);
  qr += w1 * (c10 * q3 + c11 * q2 + c12 * q1);
  qr += w2 * (c20 * q2 + c21 * q1 + c22 * q0);
  qr *= ws;
  const double ar = 3.0 * ws * w0 * w1 * w2 / (g2 * w0 * w1 + g1 * w0 * w2 + g0 * w1 * w2) + eps;
  double dq = q3 - q2;
  const double dm = q2 - q1;
  const double dc = (dm * dq > 0.0) * 0.5 * (dm + dq);
  dq = 0.5 * copysign(smin(fabs(dc), 2.0 * smin(fabs(dm), fabs(dq))), dc);
  const double alin = 2.0 * al * ar / (al + ar);
  ql = alin * ql + (1.0 - alin) * (q2 + dq);
  qr = alin * qr + (1.0 - alin) * (q2 - dq);
}

}  // namespace exact
}  // namespace pgb

#include "stencil_impl.cuh"
#include "stencil_launch.cuh"
