// Mirrors the reference header of the same path (parthenon-hpc-lab/parthenon
// src/reconstruct/dc_inline.hpp): donor-cell (first-order) face states along a row.
#pragma once
#include "../pgb_compat/all.hpp"

namespace parthenon {
// left state at face i is the cell i-1 value, right state the cell i value
template <typename T>
KOKKOS_FORCEINLINE_FUNCTION void DonorCell(const int l, const int k, const int j, const int il, const int iu,
                                           const T &q, T &ql, T &qr) {
  for (int i = il; i <= iu; ++i) {
    ql(l, i + 1) = q(l, k, j, i);
    qr(l, i) = q(l, k, j, i);
  }
}
}  // namespace parthenon
