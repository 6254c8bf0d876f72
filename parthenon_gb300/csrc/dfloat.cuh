// Double-float arithmetic: a value is an unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi)/2, about 47 significant bits, computed on the FP32 pipe.
//
// Why: GB300 issues one FP64 lane operation per SM for every 64 FP32 ones, so a stencil
// whose FP64 work is a long dependent chain of multiplies, adds and reciprocals (the
// WENO5-Z nonlinear weights) runs far faster as ~10 FP32 operations per step. The
// building blocks are the error-free transformations of Dekker ("A floating-point
// technique for extending the available precision", Numer. Math. 18, 1971) and Knuth
// (TAOCP vol. 2, 4.2.2: two-sum), with the FMA form of the exact product; the
// composite operations follow the double-double algorithms of Hida, Li and Bailey
// ("Algorithms for quad-double precision floating point arithmetic", ARITH 15, 2001)
// in their two-word form, and the reciprocal is one Newton step on a single-precision
// seed.
//
// Every operation here is a separately rounded FP32 operation written through an
// intrinsic, so that the compiler neither contracts nor reorders it (the algorithms
// depend on exact rounding of each step). The functions are also compiled for the
// host (tests check them against long double), where the build uses
// -ffp-contract=off and std::fmaf.
//
// Range: the pair keeps its precision only while lo stays a normal float, i.e. |hi|
// above about 2^-102; callers check their operands' magnitudes and take an FP64 path
// otherwise.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PGB_DF __host__ __device__ __forceinline__
#else
#include <cmath>
#define PGB_DF inline
#endif

namespace pgb {
namespace dfl {

struct df {
  float hi, lo;
};

// ---- separately rounded FP32 operations --------------------------------------------
PGB_DF float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
PGB_DF float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
PGB_DF float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
PGB_DF float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
// single-precision reciprocal seed: the hardware approximation (within 1 ulp) on the
// device, the correctly rounded quotient on the host; the Newton step in recip() squares
// its error either way
PGB_DF float frcp(float a) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
#else
  return 1.0f / a;
#endif
}

PGB_DF uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
PGB_DF float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
PGB_DF uint64_t d2u(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
#endif
}
PGB_DF double u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}

// ---- error-free transformations -----------------------------------------------------
// s + e == a + b exactly (Knuth two-sum)
PGB_DF df two_sum(float a, float b) {
  const float s = fadd(a, b);
  const float bb = fsub(s, a);
  const float e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
  return {s, e};
}
// s + e == a + b exactly when |a| >= |b| or a == 0 (Dekker fast two-sum)
PGB_DF df fast_two_sum(float a, float b) {
  const float s = fadd(a, b);
  return {s, fsub(b, fsub(s, a))};
}
// p + e == a * b exactly (FMA form)
PGB_DF df two_prod(float a, float b) {
  const float p = fmul(a, b);
  return {p, ffma(a, b, -p)};
}

// ---- double-float operations --------------------------------------------------------
PGB_DF df make(float hi) { return {hi, 0.0f}; }
PGB_DF df neg(df a) { return {-a.hi, -a.lo}; }
PGB_DF df dabs(df a) { return a.hi < 0.0f ? neg(a) : a; }
// a * 2^k for a power of two given as a float (exact)
PGB_DF df scale(df a, float pow2) { return {fmul(a.hi, pow2), fmul(a.lo, pow2)}; }

// sum with one renormalisation: error below 2^-46 (|a| + |b|), which is all the callers
// need (they use absolute, not relative, accuracy of differences)
PGB_DF df add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo = fadd(s.lo, fadd(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}
PGB_DF df sub(df a, df b) { return add(a, neg(b)); }
PGB_DF df add(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo = fadd(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}
// a + b when |a.hi| >= |b| (or a == 0): one fast two-sum instead of a two-sum
PGB_DF df add_dominant(df a, float b) {
  df s = fast_two_sum(a.hi, b);
  s.lo = fadd(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}
PGB_DF df mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = ffma(a.hi, b.lo, p.lo);
  p.lo = ffma(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
// product with a float constant
PGB_DF df mul(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = ffma(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
PGB_DF df sqr(df a) {
  df p = two_prod(a.hi, a.hi);
  p.lo = ffma(fadd(a.hi, a.hi), a.lo, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
// ---- unnormalised variants ----------------------------------------------------------
// The same sums and products without the final renormalisation: the pair's value is
// kept as accurately, but lo may exceed ulp(hi)/2 (after a cancellation hi may even be 0
// while lo is not). Sums of such pairs stay accurate. A product drops lo*lo, so its
// factors must be normalised (a larger lo costs it accuracy); sign tests, comparisons,
// reciprocals and exponent reads also need norm() first.
PGB_DF df norm(df a) { return fast_two_sum(a.hi, a.lo); }
PGB_DF df addu(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return {s.hi, fadd(s.lo, fadd(a.lo, b.lo))};
}
PGB_DF df subu(df a, df b) { return addu(a, neg(b)); }
PGB_DF df addu(df a, float b) {
  const df s = two_sum(a.hi, b);
  return {s.hi, fadd(s.lo, a.lo)};
}
PGB_DF df mulu(df a, df b) {
  const df p = two_prod(a.hi, b.hi);
  return {p.hi, ffma(a.lo, b.hi, ffma(a.hi, b.lo, p.lo))};
}
PGB_DF df mulu(df a, float b) {
  const df p = two_prod(a.hi, b);
  return {p.hi, ffma(a.lo, b, p.lo)};
}
PGB_DF df sqru(df a) {
  const df p = two_prod(a.hi, a.hi);
  return {p.hi, ffma(fadd(a.hi, a.hi), a.lo, p.lo)};
}

// 1/a: single-precision seed r, one Newton correction r + r (1 - a r) (relative error
// about 2^-45). The residual 1 - a.hi r is about 2^-23 in size, so the FMA that forms it
// rounds it with an error near 2^-47; a second FMA takes off a.lo r.
PGB_DF df recip(df a) {
  const float r = frcp(a.hi);
  const float res = ffma(-a.lo, r, ffma(-a.hi, r, 1.0f));  // 1 - a r
  return fast_two_sum(r, fmul(r, res));
}
// 1/a as above without the final renormalisation: r + r (1 - a r), whose second word is
// already within about ulp(r) (for factors of products and terms of sums)
PGB_DF df recipu(df a) {
  const float r = frcp(a.hi);
  const float res = ffma(-a.lo, r, ffma(-a.hi, r, 1.0f));
  return {r, fmul(r, res)};
}
// a / b
PGB_DF df div(df a, df b) { return mul(a, recip(b)); }

// a > b, a < b for normalised pairs
PGB_DF bool gt(df a, df b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
PGB_DF bool lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
PGB_DF df dmin(df a, df b) { return lt(b, a) ? b : a; }
PGB_DF df dmax(df a, df b) { return gt(b, a) ? b : a; }

// ---- conversions through the bit patterns (integer pipe, no FP64 instruction) ------
// The conversions take a power-of-two scale 2^off (off an integer) so that callers can
// bring a line of values to magnitudes near 1 before they enter the pairs: the pairs
// then hold every value whose scaled magnitude lies in [2^kMinExp, 2^(kMaxExp+1)).
constexpr int kMinExp = -80;
constexpr int kMaxExp = 126;

// biased binary exponent field of a double (0 for zero and subnormals)
PGB_DF int dexp_field(double x) { return (int)((d2u(x) >> 52) & 0x7ff); }

// x * 2^off as a pair. Scaled magnitudes below 2^kMinExp give 0 (an absolute error
// below 2^kMinExp of the scale); above 2^kMaxExp the pair saturates to +-FLT_MAX
// (callers choose off so that this does not happen). hi takes the leading 24
// significand bits, lo the next 29 rounded to 23: the pair holds x to a relative 2^-47.
// NORM false leaves out the final renormalisation: hi then holds the leading 24 bits
// truncated and lo the rest (|lo| <= ulp(hi), same sign as hi), an unnormalised pair
// for sums, products and sign tests.
template <bool NORM = true>
PGB_DF df from_double(double x, int off = 0) {
  const uint64_t u = d2u(x);
  const uint32_t sign = (uint32_t)(u >> 32) & 0x80000000u;
  const int ef = (int)((u >> 52) & 0x7ff);
  const int e = ef - 1023 + off;
  if (ef == 0 || e < kMinExp) return {0.0f, 0.0f};
  if (e > kMaxExp) return {u2f(sign | 0x7f7fffffu), 0.0f};
  const uint64_t m = u & 0x000fffffffffffffull;
  const float hi = u2f(sign | ((uint32_t)(e + 127) << 23) | (uint32_t)(m >> 29));
  // the remaining 29 bits rounded to their top 23 (r <= 2^23), read as an integer
  // through a float whose exponent is 2^23 (exact), then scaled by 2^(e - 46), which
  // is a normal float for e >= -80
  const uint32_t r = ((uint32_t)(m & 0x1fffffffull) + 32u) >> 6;
  const float ri = fsub(u2f(0x4b000000u + r), 8388608.0f);
  const float sc = u2f((uint32_t)(e - 46 + 127) << 23);
  const float lo = fmul(ri, sc);
  if (!NORM) return {hi, sign ? -lo : lo};
  return fast_two_sum(hi, sign ? -lo : lo);
}
// f * 2^-off as a double, exactly (zero and results below the double range give 0)
PGB_DF double f2d(float f, int off = 0) {
  const uint32_t u = f2u(f);
  const int ex = (int)((u >> 23) & 0xff);
  if (ex == 0) return 0.0;  // zero (subnormal lo parts are below the pair's precision)
  const int ed = ex - 127 + 1023 - off;
  if (ed <= 0) return 0.0;
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint64_t m = (uint64_t)(u & 0x7fffffu) << 29;
  if (ed >= 2047) return u2d(sign | 0x7ff0000000000000ull);
  return u2d(sign | ((uint64_t)ed << 52) | m);
}
// a * 2^-off as a double: one FP64 add of the two exact halves
PGB_DF double to_double(df a, int off = 0) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(f2d(a.hi, off), f2d(a.lo, off));
#else
  return f2d(a.hi, off) + f2d(a.lo, off);
#endif
}
// 2^-off as a double for to_double_pow2 (off in [-1022, 1022]; callers check)
PGB_DF double pow2d_neg(int off) { return u2d((uint64_t)(1023 - off) << 52); }
// a * 2^-off as a double with the hardware conversions: the two halves convert
// exactly, their FP64 sum is exact (about 48 significant bits), and the product with
// the power of two is exact while the result stays a normal double
PGB_DF double to_double_pow2(df a, double pow2) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(__dadd_rn((double)a.hi, (double)a.lo), pow2);
#else
  return ((double)a.hi + (double)a.lo) * pow2;
#endif
}
// 2^k as a float: 0 below the normal range, +inf above it
PGB_DF float pow2f(int k) {
  const int ex = k + 127;
  return ex <= 0 ? 0.0f : (ex >= 255 ? u2f(0x7f800000u) : u2f((uint32_t)ex << 23));
}
// a double constant as a pair, evaluated at compile time
constexpr df constant(double x) { return {(float)x, (float)(x - (double)(float)x)}; }

}  // namespace dfl
}  // namespace pgb
