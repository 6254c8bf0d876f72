// Host build of the fast Burgers sweep's per-cell reconstruction (weno_df.cuh): marches
// one line of cell values exactly as the kernel does (double-float step, FP64
// reference expression for lanes outside the pairs' range) so the CPU tests can
// compare it with the reference formula over many lines. Test infrastructure only.
#include <algorithm>

#include "../../parthenon_gb300/csrc/weno_df.cuh"

using namespace pgb;

extern "C" {

// q: m cell values; writes ql[p], qr[p] for p = 2 .. m-3 (others untouched) and returns
// the number of cells that took the FP64 expression.
int pgb_test_weno_line(const double *q, int m, double *ql, double *qr) {
  if (m < 5) return -1;
  int emax = 0;
  for (int i = 0; i < m; ++i) emax = std::max(emax, dfl::dexp_field(q[i]));
  const int off = wdf::line_offset(emax);
  wdf::Line w;
  wdf::prime(w, q[0], q[1], q[2], q[3], off);
  int nfb = 0;
  for (int p = 2; p <= m - 3; ++p) {
    dfl::df l, r;
    if (!wdf::step(w, q[p + 2], l, r)) {
      double a, b;
      wdf::weno5z_ref(q[p - 2], q[p - 1], q[p], q[p + 1], q[p + 2], a, b);
      l = dfl::from_double(a, off);
      r = dfl::from_double(b, off);
      ++nfb;
    }
    ql[p] = dfl::to_double(l, off);
    qr[p] = dfl::to_double(r, off);
  }
  return nfb;
}

// the FP64 reference expression on the same cells (for checking the restatement)
void pgb_test_weno_ref(const double *q, int m, double *ql, double *qr) {
  for (int p = 2; p <= m - 3; ++p) wdf::weno5z_ref(q[p - 2], q[p - 1], q[p], q[p + 1], q[p + 2], ql[p], qr[p]);
}

// double -> pair -> double round trip (normalised pair, or the unnormalised conversion
// when raw != 0)
double pgb_test_df_roundtrip(double x) { return dfl::to_double(dfl::from_double(x)); }
double pgb_test_df_roundtrip_raw(double x) { return dfl::to_double(dfl::from_double<false>(x)); }
// the increment conversion through 2^-off (hardware conversions on the device)
double pgb_test_df_pow2(double x, int off) {
  return dfl::to_double_pow2(dfl::from_double(x, off), dfl::pow2d_neg(off));
}

// pair arithmetic on converted inputs, returned as doubles: op 0 add, 1 sub, 2 mul,
// 3 div, 4 recip(a), 5 sqr(a), 6 recipu(a) (unnormalised reciprocal), 7 mulu(a, recipu(b))
// (a quotient through the unnormalised forms)
double pgb_test_df_op(int op, double a, double b) {
  const dfl::df x = dfl::from_double(a), y = dfl::from_double(b);
  switch (op) {
    case 0: return dfl::to_double(dfl::add(x, y));
    case 1: return dfl::to_double(dfl::sub(x, y));
    case 2: return dfl::to_double(dfl::mul(x, y));
    case 3: return dfl::to_double(dfl::div(x, y));
    case 4: return dfl::to_double(dfl::recip(x));
    case 5: return dfl::to_double(dfl::sqr(x));
    case 6: return dfl::to_double(dfl::recipu(x));
    case 7: return dfl::to_double(dfl::mulu(x, dfl::recipu(y)));
    default: return 0.0;
  }
}

}  // extern "C"
