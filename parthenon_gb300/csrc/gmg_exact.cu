// Multigrid kernels, exact build: -fmad=false and the reference's expression order, so
// an FP64 V-cycle is bitwise identical to the CPU restatement.
#define PGB_GMG_NS gmg_exact
#define PGB_GMG_EXACT 1
#include "gmg_impl.cuh"

namespace pgb {
namespace gmg_exact {
void vcycle_d(GmgLevelBuf<double> *L, int nl, const GmgConfig &c, cudaStream_t s) { vcycle<double>(L, nl, c, nullptr, s); }
void residual_sumsq_d(GmgLevelBuf<double> &L, const GmgConfig &c, double *partial, int np, double *res, float *rhs32,
                      cudaStream_t s) {
  residual_sumsq<double>(L, c, partial, np, res, rhs32, s);
}
void apply_d(const GmgLevelBuf<double> &L, const GmgConfig &c, const double *u, double *out, cudaStream_t s) {
  apply<double>(L, c, u, out, s);
}
}  // namespace gmg_exact
}  // namespace pgb
