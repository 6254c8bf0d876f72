// Multigrid level storage and configuration shared by the GMG builds and the C ABI.
#pragma once

#include <cstdint>

namespace pgb {

struct GmgConfig {
  int stages = 2;        // smoother sweeps per pre/post smooth
  int jacobi = 0;        // 0: SRJ weights for `stages`; 1: weighted Jacobi with `weight`
  double weight = 2.0 / 3.0;
  int coarse_sweeps = 0; // extra smoother passes at the coarsest level
  double D = 1.0, alpha = 0.0;
};

// One level: n^3 cells, x fastest, periodic. All arrays are device memory.
template <class T>
struct GmgLevelBuf {
  int n = 0, log2n = 0;
  double dx = 0, xmin = 0;
  T *u = nullptr, *rhs = nullptr, *res = nullptr, *temp = nullptr, *u0 = nullptr;
  int64_t cells() const { return (int64_t)n * n * n; }
};

}  // namespace pgb
