// Multigrid kernels, fast build: FMA contraction and the constant-coefficient operator as
// a 7-point Laplacian. Serves the FP64 V-cycle and the FP32 V-cycle of the mixed-
// precision solve (FP64 residual and update, FP32 V-cycle, FP64 coarsest level).
#define PGB_GMG_NS gmg_fast
#include "gmg_impl.cuh"

namespace pgb {
namespace gmg_fast {
void vcycle_d(GmgLevelBuf<double> *L, int nl, const GmgConfig &c, cudaStream_t s) { vcycle<double>(L, nl, c, nullptr, s); }
void vcycle_f(GmgLevelBuf<float> *L, int nl, const GmgConfig &c, GmgLevelBuf<double> *c64, cudaStream_t s) {
  vcycle<float>(L, nl, c, c64, s);
}
void residual_sumsq_d(GmgLevelBuf<double> &L, const GmgConfig &c, double *partial, int np, double *res, float *rhs32,
                      cudaStream_t s) {
  residual_sumsq<double>(L, c, partial, np, res, rhs32, s);
}
void apply_d(const GmgLevelBuf<double> &L, const GmgConfig &c, const double *u, double *out, cudaStream_t s) {
  apply<double>(L, c, u, out, s);
}
void mixed_prepare(const double *r64, GmgLevelBuf<float> &L0, cudaStream_t s) { launch_mixed_prepare(r64, L0, s); }
void mixed_update(double *x, const GmgLevelBuf<float> &L0, cudaStream_t s) { launch_mixed_update(x, L0, s); }
}  // namespace gmg_fast
}  // namespace pgb
