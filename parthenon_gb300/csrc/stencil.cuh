// Finite-volume stencil kernels: reconstruction + Riemann flux + flux difference +
// low-storage RK update, marching along one direction per launch.
//
// Each thread owns one line of cells along direction D (fixed transverse indices) and
// walks it from the first ghost face to the last. At every cell it reconstructs all
// components once (each cell's WENO/PLM is evaluated exactly once per direction, as
// in the reference), forms the flux at the face it shares with the previous cell, and
// emits that previous cell's flux difference. Nothing is recomputed and every lane of
// a warp does the same work, which matters because the FP64 pipe (not HBM) bounds
// these kernels on GB300.
//
// Reference semantics (parthenon-hpc-lab/parthenon):
//   benchmarks/burgers/burgers_package.cpp:202-404, burgers_package.hpp:32-43,
//   benchmarks/burgers/recon.hpp:27-99                 Burgers fluxes
//   example/advection/advection_package.cpp:499-647,
//   src/reconstruct/dc_inline.hpp, plm_inline.hpp      advection fluxes
//   src/interface/update.hpp:42-56, update.cpp:62-85   flux divergence
//   src/interface/update.hpp:70-136                    Average / Update weighted sums
//
// The flux difference for a cell is accumulated across the three directional launches
// in the reference's order: du = x-term; du += y-term; du += z-term; dudt = -du/V.
#pragma once

#include <cfloat>

#include "common.cuh"

namespace pgb {

constexpr double kWenoEps = 10 * DBL_EPSILON;

// Output modes of a directional launch.
enum StencilMode : int {
  kStoreDu = 0,      // dudt  = du_D
  kAddDu = 1,        // dudt += du_D
  kFinishUpdate = 2, // du = dudt + du_D; out = (w_in*u_in + w_base*u_base) + beta_dt*(-du/V)
  kStoreFlux = 3,    // flux arrays only (multilevel path)
  kFinishUpdateFromSingle = 4,  // single direction meshes: du = du_D then update
};

struct StageArgs {
  const double *u_in;    // state the fluxes are computed from (mc0)
  const double *u_base;  // base state for the RK average
  double *u_out;         // updated state (mc1), interior only
  double *dudt;          // accumulator [block][comp][N3][N2][N1] (interior used)
  double *flux;          // flux arrays [block][dir][comp][N3][N2][N1] (kStoreFlux)
  const double *dt;      // device scalar: current time step
  double w_in, w_base;   // Average weights (beta, 1 - beta)
  double beta;           // Update weight (dt factor)
  const DevBlockGeom *geom;
  Dims d;
  int nblocks;           // blocks this launch covers
  const int *blist;      // their indices (null: blocks 0 .. nblocks - 1)
  int tune_nblocks;      // the mesh's blocks and multilevel flag: the autotuner's key
  int tune_ml;           // (one choice per mesh for every launch of its stage)
  int recon;             // Burgers: 0 WENO5, 1 linear; advection: 0 donor cell, 1 PLM
  double vel[3];         // advection velocity
  int ncomp;             // components of the fields
  int ncvel;             // advection: 0, or one velocity per component in cvel
  double cvel[16][3];
  const uint8_t *alloc;  // sparse variables: [block * ncomp + v] allocated (null: dense)
};

}  // namespace pgb
