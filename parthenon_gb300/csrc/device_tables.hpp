// Flat, device-resident descriptor tables for the block-AMR kernels.
//
// The host topology (topology.hpp) is lowered once per mesh (re-lowered on remesh)
// into these POD arrays. Kernels are driven only by them: no pointers to host
// structures, no per-call host work, so a whole stage can be captured in a CUDA graph.
#pragma once

#include <cstdint>

namespace pgb {

// Box of cells: start (i,j,k) and extents (ni,nj,nk).
struct DevBox {
  int32_t lo[3];
  int32_t n[3];
};

// Ghost copy between two blocks. Element m of the send box (row-major over
// (component, k, j, i)) lands on element m of the receive box when `mask` allows it.
struct DevPair {
  int32_t src_block, dst_block;
  int32_t src_coarse, dst_coarse;  // 1 = coarse buffer of the block
  DevBox src, dst;
  uint32_t mask;                   // 27-bit ownership mask of the receive box
  int32_t full_mask;               // 1 when every element of the box is active
  int64_t buf_off;                 // element offset of this pair in the packed buffer
};

// A unit of work: `nrows` rows (component, k, j) of one pair / region, from `row0`.
struct DevWork {
  int32_t item;
  int32_t row0;
  int32_t nrows;
  int32_t pad;
};

// Restriction or prolongation region in coarse index space of one block.
struct DevRegion {
  int32_t block;
  DevBox box;
  uint32_t mask;
  int32_t full_mask;
};

// Flux correction of one fine/coarse face: fine block restricts face fluxes over
// `fine` (coarse face index space) and writes them into the coarse block over `recv`.
struct DevFluxCorr {
  int32_t fine_block, coarse_block, dir, pad;
  DevBox fine, recv;
  uint32_t mask;
  int32_t full_mask;
};

// Per-block geometry used by stencil kernels and prolongation.
struct DevBlockGeom {
  double xmin[3];  // coordinate of index 0 (ghost included) cell face, fine grid
  double dx[3];
  double area[3];
  double vol;
  double cxmin[3];  // coarse-buffer grid
  double cdx[3];
};

struct Dims {
  int32_t N[3];   // fine block arrays with ghosts
  int32_t Nc[3];  // coarse buffers with ghosts
  int32_t ng;
  int32_t nx[3];  // interior cells
};

// Sparse-variable state seen by the kernels (one variable per field component).
struct SparseDev {
  uint8_t *alloc;      // [block * ncomp + v]: variable allocated on the block
  int32_t *count;      // [block * ncomp + v]: consecutive all-below deallocation checks
  uint8_t *recv;       // [block * ncomp + v]: data received this exchange (allocate)
  uint8_t *pair_flag;  // [pair * ncomp + v]: the pair's buffer carries data (else null)
  uint8_t *fc_flag;    // [flux correction * ncomp + v]: the fine side sends
  const double *thr;   // [3][ncomp]: allocation threshold, deallocation threshold, default
  int32_t ncomp;
  int32_t dealloc_count;
};

// Containers whose (block, variable) slices are zeroed when a variable is deallocated.
struct ZeroList {
  double *cell[4];     // [block][ncomp][N3][N2][N1]
  double *coarse[2];   // [block][ncomp][Nc3][Nc2][Nc1]
  double *flux;        // [block][3][ncomp][N3][N2][N1]
  int32_t ncell, ncoarse;
};

__host__ __device__ inline bool mask_active(uint32_t mask, const DevBox &b, int k, int j, int i) {
  const int ii = (i == b.lo[0] + b.n[0] - 1) - (i == b.lo[0]);
  const int jj = (j == b.lo[1] + b.n[1] - 1) - (j == b.lo[1]);
  const int kk = (k == b.lo[2] + b.n[2] - 1) - (k == b.lo[2]);
  return (mask >> ((ii + 1) + 3 * (jj + 1) + 9 * (kk + 1))) & 1u;
}

}  // namespace pgb
