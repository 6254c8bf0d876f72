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

// Team versions on one row (k, j) of a pack, for every variable: X1 puts cell i's value
// in the left state of face i+1 and the right state of face i; X2 and X3 put it in both
// states at index i (the caller passes the row below for the left states).
template <typename T>
KOKKOS_FORCEINLINE_FUNCTION void DonorCellX1(team_mbr_t const &member, const int k, const int j, const int il,
                                             const int iu, const T &q, ScratchPad2D<Real> &ql,
                                             ScratchPad2D<Real> &qr) {
  const int nvar = q.GetDim(4);
  for (int n = 0; n < nvar; ++n)
    par_for_inner(member, il, iu, [&](const int i) {
      const Real v = q(n, k, j, i);
      ql(n, i + 1) = v;
      qr(n, i) = v;
    });
}
template <typename T>
KOKKOS_FORCEINLINE_FUNCTION void DonorCellX2(team_mbr_t const &member, const int k, const int j, const int il,
                                             const int iu, const T &q, ScratchPad2D<Real> &ql,
                                             ScratchPad2D<Real> &qr) {
  const int nvar = q.GetDim(4);
  for (int n = 0; n < nvar; ++n)
    par_for_inner(member, il, iu, [&](const int i) {
      const Real v = q(n, k, j, i);
      ql(n, i) = v;
      qr(n, i) = v;
    });
}
template <typename T>
KOKKOS_FORCEINLINE_FUNCTION void DonorCellX3(team_mbr_t const &member, const int k, const int j, const int il,
                                             const int iu, const T &q, ScratchPad2D<Real> &ql,
                                             ScratchPad2D<Real> &qr) {
  DonorCellX2(member, k, j, il, iu, q, ql, qr);
}
}  // namespace parthenon
