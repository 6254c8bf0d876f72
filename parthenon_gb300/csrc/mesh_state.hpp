// The library's mesh object: host topology plus its lowered device tables.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "device_tables.hpp"
#include "topology.hpp"

namespace pgb {

// Device copy of one grid's tables (the leaf grid, or one multigrid level).
struct GridTables {
  int nblocks = 0;
  Dims dims{};
  bool multilevel = false;
  int npairs = 0, ncopy_work = 0;
  int nrs = 0, nrs_work = 0;    // send-side restriction
  int nrr = 0, nrr_work = 0;    // receive-side restriction
  int npro = 0, npro_work = 0;  // prolongation
  int nfc = 0, nfc_work = 0;    // flux correction
  int64_t buffer_elems = 0;     // sum of pair box sizes (one component)
  DevPair *pairs = nullptr;
  DevWork *copy_work = nullptr;
  DevRegion *rs = nullptr, *rr = nullptr, *pro = nullptr;
  DevWork *rs_work = nullptr, *rr_work = nullptr, *pro_work = nullptr;
  DevFluxCorr *fc = nullptr;
  DevWork *fc_work = nullptr;
  // multilevel meshes: the blocks with a fine/coarse face (either side of a flux
  // correction) and the others, whose stage needs no stored fluxes
  int nfcb = 0, nplain = 0;
  int *fcb = nullptr, *plain = nullptr;
  DevBlockGeom *geom = nullptr;
  void *arena = nullptr;        // one device allocation holding every table above
  std::vector<DevBlockGeom> geom_h;
  void release();
};

// Sparse variables of a mesh (Metadata::Sparse, one field component each): per block
// an allocation flag and a deallocation counter, per variable the thresholds and the
// default value. The device arrays exist while the mesh is uploaded; the host copies
// carry the state from one mesh to the next across a remesh.
struct SparseState {
  bool on = false;
  int ncomp = 0;
  int dealloc_count = 5;
  std::vector<double> thr_h;       // [3][ncomp]: allocation, deallocation, default
  std::vector<uint8_t> alloc_h;    // staged flags [nblocks * ncomp]
  std::vector<int32_t> count_h;    // staged counters
  bool staged = false;             // host copies to be uploaded with the mesh tables
  SparseDev dev{};                 // device arrays (null until uploaded)
  void *arena = nullptr;           // the one allocation holding them
  void release();
};

struct MeshState {
  std::unique_ptr<MeshTopology> topo;
  GridTables leaf;
  bool uploaded = false;
  // device scratch owned by the mesh (reductions, status words)
  double *d_scalars = nullptr;      // [0] dt, [1] reduction scratch ...
  unsigned long long *d_minbits = nullptr;
  int *d_status = nullptr;
  std::vector<int> deref_count;     // per leaf block, MeshRefinement::deref_count_
  // Burgers "derived" field (one component, field layout) that the RK2 cycles fill after
  // every stage's update (pgb_set_derived); null: FillDerived is not run
  double *derived = nullptr;
  SparseState sparse;
  // device view for the kernels, or null when the mesh has no sparse variables
  const SparseDev *sparse_dev() const { return sparse.on && sparse.dev.alloc ? &sparse.dev : nullptr; }
  ~MeshState();
};

// sparse.cu: (re)create the device arrays of m.sparse for the uploaded tables
int sparse_upload(MeshState &m);

int lower_grid(const GridTopology &g, const MeshSpec &spec, GridTables &out, bool dry_run = false);

}  // namespace pgb
