// WENO5-Z with MC blending (benchmarks/burgers/recon.hpp:42-99) marched along a line
// in double-float arithmetic (dfloat.cuh), for the fast build of the Burgers sweep.
//
// Per cell the reference evaluates smoothness indicators beta_k (+ eps, eps = 10
// DBL_EPSILON), tau = |beta2 - beta0|, nonlinear weights alpha_k = g_k (beta_k + tau) /
// beta_k + eps, two normalisations, the blending coefficients alpha_l, alpha_r and
// their harmonic mean. This file evaluates the same quantities from exact algebraic
// rewrites:
//   B_k = 1 + tau / beta_k, left weights (g0 B0, g1 B1, g2 B2) + eps, right
//   (g0 B2, g1 B1, g2 B0) + eps;
//   the reference's D = g2 a0 a1 + g1 a0 a2 + g0 a1 a2 and a0 a1 a2 are, up to the
//   weights' eps, g0 g1 g2 E2 and g0 g1 g2 E3 with E2 = B0B1 + B0B2 + B1B2 and
//   E3 = B0B1B2, the same on both sides, so alpha_l = 3 E3 / (E2 S_L) + eps,
//   alpha_r = 3 E3 / (E2 S_R) + eps, and their harmonic mean, without the eps terms,
//   alpha_lin = 6 E3 / (E2 (S_L + S_R));
// and forms the face values about the cell value q2 from first differences
// e_k = q[k+1] - q[k]: ql = q2 + dq + alin (XL - dq), qr = q2 - dq + alin (XR + dq),
// XL = sum w_k (P_k - q2). Only the new difference e3 = q4 - q3 is an FP64 operation;
// the rest runs on the FP32 pipe.
//
// Each line is scaled by a power of two 2^off that brings its largest magnitude near 1
// (the caller finds it), so every quantity fits the float exponent range whatever the
// field's units; values below 2^-80 of the line's largest enter as zero. A cell falls
// back to the reference expression in FP64 (weno5z_ref, the caller's job) when tau > 0
// and its smallest smoothness indicator lies below 2^-40 tau (a sub-stencil that is
// exactly constant next to a jump): B_k = 1 + tau / beta_k would then exceed 2^40 and
// take the products below out of the float range.
#pragma once

#include "dfloat.cuh"

namespace pgb {
namespace wdf {

using dfl::df;

constexpr df kG0 = dfl::constant(0.1);
constexpr df kG1 = dfl::constant(0.6);
constexpr df kG2 = dfl::constant(0.3);
constexpr df kThirteenThirds = dfl::constant(13.0 / 3.0);
// the reference's eps (robust.hpp EPS(): 10 DBL_EPSILON); as a float its relative error
// (3e-8) changes sums with terms >= eps by less than 1e-22 of the term
constexpr double kEpsD = 10.0 * 2.220446049250313080847e-16;
constexpr float kEpsF = (float)kEpsD;

PGB_DF double dsub(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}

// Power-of-two scale 2^off that brings the largest magnitude of a line of values into
// [1, 2): off from the largest biased exponent field among them (0 for an all-zero line).
PGB_DF int line_offset(int max_exp_field) { return max_exp_field == 0 ? 0 : 1023 - max_exp_field; }

// Marching state of one line: cell p's stencil q[p-2..p+2], values scaled by 2^off.
struct Line {
  double q3d;     // q[p+1] in FP64, unscaled (the next difference is formed in FP64)
  df q2, q3;      // q[p], q[p+1]
  df e0, e1, e2;  // q[p-1]-q[p-2], q[p]-q[p-1], q[p+1]-q[p]
  df t2a, t2b;    // (13/3) (second difference)^2 + eps of cells p-1 and p
  int off;        // scale exponent of the line
  float eps_b;    // the smoothness indicators' eps in scaled units (eps 2^(2 off))
  bool eps_only;  // eps exceeds every scaled indicator by far: B_k = 1 exactly
};

// (13/3) d2^2 + eps (the indicators' eps rides with the term each cell's three
// indicators share along the line), feeding sums only: left unnormalised
PGB_DF df t2_of(df d2, float eps_b) { return dfl::addu(dfl::mulu(dfl::sqru(d2), kThirteenThirds), eps_b); }

// Prime with q[p-2], q[p-1], q[p], q[p+1] of the first cell p and the line's scale.
PGB_DF void prime(Line &w, double q0, double q1, double q2, double q3, int off) {
  const double e0 = dsub(q1, q0), e1 = dsub(q2, q1), e2 = dsub(q3, q2);
  w.off = off;
  // eps 2^(2 off): beyond the float range above (a line of magnitude below 2^-88,
  // whose indicators are then below eps 2^-80 and leave B_k = 1 in FP64 too), below it
  // negligible against indicators of order one
  w.eps_only = 2 * off > 175;
  w.eps_b = w.eps_only ? 0.0f : dfl::fmul(kEpsF, dfl::pow2f(2 * off));
  w.q3d = q3;
  w.q2 = dfl::from_double(q2, off);
  w.q3 = dfl::from_double(q3, off);
  w.e0 = dfl::from_double(e0, off);
  w.e1 = dfl::from_double(e1, off);
  w.e2 = dfl::from_double(e2, off);
  w.t2a = t2_of(dfl::sub(w.e1, w.e0), w.eps_b);
  w.t2b = t2_of(dfl::sub(w.e2, w.e1), w.eps_b);
}

// Face values of cell p (ql at its right face, qr at its left face, scaled, as
// unnormalised pairs) given
// q[p+2], then advance the window by one cell. Returns false when this cell must be
// evaluated in FP64 instead (the window still advances).
PGB_DF bool step(Line &w, double q4, df &ql, df &qr) {
  using namespace dfl;
  const double e3d = dsub(q4, w.q3d);
  // e3 is compared (as e1, e2) in the MC limiter against normalised pairs, which needs
  // it normalised; q4 enters sums only
  const df e3 = from_double(e3d, w.off);
  const df q4p = from_double<false>(q4, w.off);
  const df e0 = w.e0, e1 = w.e1, e2 = w.e2;
  // Sums and the products that only feed sums keep their pairs unnormalised
  // (dfloat.cuh addu/mulu/sqru/recipu); a pair that enters a sign test or a comparison
  // is normalised first (after a cancellation a pair holds its value in lo). Products
  // also take unnormalised factors (the first-difference combinations b0, b2 and d*,
  // the second difference of t2, B_k, the weight sums, E2, E3, the reciprocals, the
  // weighted sums and the blend's differences): a product drops lo*lo, which is at most
  // 2^-46 of the product when lo is within a few ulp of hi, and after a cancellation
  // (hi near zero, the value in lo) is below 2^-46 of the differences that cancelled; a
  // reciprocal's Newton step takes an unnormalised argument the same way. Face values
  // stay within 1.8e-14 of the line's magnitude over the host test's random lines (its
  // bar is 3e-14; 99.9% of faces within 1.2e-14); leaving B1 B2, the blending
  // coefficient's last product and the sum under its reciprocal unnormalised as well
  // took the worst face to 2.7-3.0e-14, so those stay normalised.
  // smoothness indicators (recon.hpp:54-64 in first differences)
  const df t2c = t2_of(subu(e3, e2), w.eps_b);
  const df b0 = subu(mulu(e1, 3.0f), e0);
  const df b1 = norm(addu(e1, e2));
  const df b2 = subu(e3, mulu(e2, 3.0f));
  const df be0 = addu(sqru(b0), w.t2a);
  const df be1 = addu(sqru(b1), w.t2b);
  const df be2 = addu(sqru(b2), t2c);
  const df tau = dabs(norm(subu(be2, be0)));
  bool fast = true;
  df B0 = make(1.0f), B1 = make(1.0f), B2 = make(1.0f);
  if (tau.hi != 0.0f && !w.eps_only) {
    // B_k = 1 + tau / beta_k; a B_k above 2^40 (a zero indicator included) would take
    // the products below out of the float range
    fast = fminf(fminf(be0.hi, be1.hi), be2.hi) >= fmul(tau.hi, 0x1p-40f);
    B0 = addu(mulu(tau, recipu(be0)), 1.0f);
    B1 = addu(mulu(tau, recipu(be1)), 1.0f);
    B2 = addu(mulu(tau, recipu(be2)), 1.0f);
  }
  // nonlinear weights g_k B_k + eps (unnormalised) and their sums: g_k B_k >= 0.1, whose
  // float ulp (2^-27) is far above eps (2e-15), so eps belongs to the low word alone
  const auto weight = [](df B, df g) {
    const df m = mulu(B, g);
    return df{m.hi, fadd(m.lo, kEpsF)};
  };
  const df l0 = weight(B0, kG0), l1 = weight(B1, kG1), l2 = weight(B2, kG2);
  const df r0 = weight(B2, kG0), r2 = weight(B0, kG2);
  const df SL = addu(addu(l0, l1), l2);
  const df SR = addu(addu(r0, l1), r2);
  const df isL = recipu(SL), isR = recipu(SR);
  // blending coefficients alpha_l = 3 E3/(E2 S_L) + eps, alpha_r likewise, and their
  // harmonic mean alpha_lin = 2 al ar / (al + ar): without the two eps terms this is
  // 6 E3 / (E2 (S_L + S_R)); leaving them out moves alpha_lin by about eps, i.e. the
  // face value by about eps times the stencil's differences. a6 = alpha_lin / 6 (the
  // candidate polynomials below carry the 6)
  const df B12 = mul(B1, B2);
  const df E2 = addu(mulu(B0, addu(B1, B2)), B12);
  const df E3 = mulu(B0, B12);
  const df a6 = mul(E3, recipu(mul(E2, add(SL, SR))));
  // 6 (P_k - q2) for the candidate polynomials of both faces (recon.hpp:45-47,69-85)
  const df d0 = subu(mulu(e1, 5.0f), scale(e0, 2.0f));
  const df d1 = addu(e1, scale(e2, 2.0f));
  const df d2 = subu(scale(e2, 4.0f), e3);
  const df d0r = subu(scale(e3, 2.0f), mulu(e2, 5.0f));
  const df d1r = neg(addu(scale(e1, 2.0f), e2));
  const df d2r = subu(e0, scale(e1, 4.0f));
  // 6 XL, 6 XR: the weighted sums of 6 (P_k - q2)
  const df XL6 = mulu(addu(addu(mulu(l0, d0), mulu(l1, d1)), mulu(l2, d2)), isL);
  const df XR6 = mulu(addu(addu(mulu(r0, d0r), mulu(l1, d1r)), mulu(r2, d2r)), isR);
  // MC-limited slope (recon.hpp:27-40, 87-88): dq = sign(s) min(|s|/4, |e1|, |e2|) when
  // e1 and e2 have the same sign (both nonzero), else 0; s = e1 + e2 = b1
  const bool same = (e1.hi > 0.0f && e2.hi > 0.0f) || (e1.hi < 0.0f && e2.hi < 0.0f);
  const df mag = dmin(scale(dabs(b1), 0.25f), dmin(dabs(e1), dabs(e2)));
  df dq = b1.hi < 0.0f ? neg(mag) : mag;
  if (!same) dq = make(0.0f);
  // blend (recon.hpp:90-92) about q2: alpha_lin (XL - dq) = a6 (6 XL - 6 dq)
  // the face values come back unnormalised: they feed flux products and sums (a
  // caller that compares them normalises first; norm() does not change a pair's value)
  const df dq6 = mulu(dq, 6.0f);
  ql = addu(w.q2, addu(dq, mulu(a6, subu(XL6, dq6))));
  qr = addu(w.q2, subu(mulu(a6, addu(XR6, dq6)), dq));
  // advance
  w.q3d = q4;
  w.q2 = w.q3;
  w.q3 = q4p;
  w.e0 = e1;
  w.e1 = e2;
  w.e2 = e3;
  w.t2a = w.t2b;
  w.t2b = t2c;
  return fast;
}

// The reference expression (recon.hpp:42-99) in FP64, separately rounded in its order:
// the fallback of lanes outside the pair's range.
PGB_DF void weno5z_ref(double q0, double q1, double q2, double q3, double q4, double &ql, double &qr) {
#if defined(__CUDA_ARCH__)
#define PGB_M(a, b) __dmul_rn(a, b)
#define PGB_A(a, b) __dadd_rn(a, b)
#define PGB_S(a, b) __dsub_rn(a, b)
#define PGB_D(a, b) __ddiv_rn(a, b)
#else
#define PGB_M(a, b) ((a) * (b))
#define PGB_A(a, b) ((a) + (b))
#define PGB_S(a, b) ((a) - (b))
#define PGB_D(a, b) ((a) / (b))
#endif
  const double eps = kEpsD;
  const double tt = 13.0 / 3.0;
  const double a0 = PGB_A(PGB_S(q0, PGB_M(2.0, q1)), q2);
  const double c0 = PGB_A(PGB_S(q0, PGB_M(4.0, q1)), PGB_M(3.0, q2));
  double be0 = PGB_A(PGB_A(PGB_M(PGB_M(tt, a0), a0), PGB_M(c0, c0)), eps);
  const double a1 = PGB_A(PGB_S(q1, PGB_M(2.0, q2)), q3);
  const double c1 = PGB_S(q3, q1);
  double be1 = PGB_A(PGB_A(PGB_M(PGB_M(tt, a1), a1), PGB_M(c1, c1)), eps);
  const double a2 = PGB_A(PGB_S(q2, PGB_M(2.0, q3)), q4);
  const double c2 = PGB_A(PGB_S(q4, PGB_M(4.0, q3)), PGB_M(3.0, q2));
  double be2 = PGB_A(PGB_A(PGB_M(PGB_M(tt, a2), a2), PGB_M(c2, c2)), eps);
  const double tau = fabs(PGB_S(be2, be0));
  be0 = PGB_D(PGB_A(be0, tau), be0);
  be1 = PGB_D(PGB_A(be1, tau), be1);
  be2 = PGB_D(PGB_A(be2, tau), be2);
  auto side = [&](double b0, double b1, double b2, double p0, double p1, double p2, double &out) {
    const double w0 = PGB_A(PGB_M(0.1, b0), eps);
    const double w1 = PGB_A(PGB_M(0.6, b1), eps);
    const double w2 = PGB_A(PGB_M(0.3, b2), eps);
    const double ws = PGB_D(1.0, PGB_A(PGB_A(w0, w1), w2));
    double x = PGB_M(w0, p0);
    x = PGB_A(x, PGB_M(w1, p1));
    x = PGB_A(x, PGB_M(w2, p2));
    out = PGB_M(x, ws);
    const double den = PGB_A(PGB_A(PGB_M(PGB_M(0.3, w0), w1), PGB_M(PGB_M(0.6, w0), w2)), PGB_M(PGB_M(0.1, w1), w2));
    return PGB_A(PGB_D(PGB_M(PGB_M(PGB_M(PGB_M(3.0, ws), w0), w1), w2), den), eps);
  };
  auto poly = [&](double x, double y, double z, double cx, double cy, double cz) {
    return PGB_A(PGB_A(PGB_M(cx, x), PGB_M(cy, y)), PGB_M(cz, z));
  };
  double xl, xr;
  const double al = side(be0, be1, be2, poly(q0, q1, q2, 1.0 / 3.0, -7.0 / 6.0, 11.0 / 6.0),
                         poly(q1, q2, q3, -1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0),
                         poly(q2, q3, q4, 1.0 / 3.0, 5.0 / 6.0, -1.0 / 6.0), xl);
  const double ar = side(be2, be1, be0, poly(q4, q3, q2, 1.0 / 3.0, -7.0 / 6.0, 11.0 / 6.0),
                         poly(q3, q2, q1, -1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0),
                         poly(q2, q1, q0, 1.0 / 3.0, 5.0 / 6.0, -1.0 / 6.0), xr);
  // MC slope (recon.hpp:27-33)
  const double dm = PGB_S(q2, q1), dp = PGB_S(q3, q2);
  const double dc = PGB_M(PGB_M((PGB_M(dm, dp) > 0.0) ? 1.0 : 0.0, 0.5), PGB_A(dm, dp));
  const double mn = fabs(dm) < fabs(dp) ? fabs(dm) : fabs(dp);
  const double lim = fabs(dc) < PGB_M(2.0, mn) ? fabs(dc) : PGB_M(2.0, mn);
  const double dq = PGB_M(0.5, copysign(lim, dc));
  const double alin = PGB_D(PGB_M(PGB_M(2.0, al), ar), PGB_A(al, ar));
  const double om = PGB_S(1.0, alin);
  ql = PGB_A(PGB_M(alin, xl), PGB_M(om, PGB_A(q2, dq)));
  qr = PGB_A(PGB_M(alin, xr), PGB_M(om, PGB_S(q2, dq)));
#undef PGB_M
#undef PGB_A
#undef PGB_S
#undef PGB_D
}

}  // namespace wdf
}  // namespace pgb
