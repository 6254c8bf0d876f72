// Ghost exchange through a buffer that the library owns in static device memory.
//
// Some callers of this library cannot allocate device memory themselves: code that runs
// while another framework owns every device allocation (a host application with its
// own pooling allocator that forbids direct cudaMalloc), or a time-critical loop where
// an allocation's latency and possible failure mid-run are not acceptable. For them
// this entry point runs the reference-layout (packed-buffer) exchange without any
// allocation: the pack buffer is a fixed array in device global memory that exists
// for as long as the library is loaded.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"
#include "mesh_state.hpp"

namespace pgb {

int exchange_grid(GridTables &t, double *fine, double *coarse, int ncomp, int prolongate, int prolong_op,
                  double *buffer, cudaStream_t s, const SparseDev *sp);
GridTables *mesh_leaf_tables(pgb_mesh *m);
MeshState *mesh_state(pgb_mesh *m);

namespace {

// Maximum packed-buffer size: 4,194,304 doubles (32 MiB). Every GPU that loads the
// library keeps this array resident until the process exits.
constexpr size_t kStaticPackDoubles = size_t(1) << 22;
static __device__ __align__(256) double g_static_pack[kStaticPackDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
double *g_static_ptr[kMaxDevices] = {};

// The host-side name `g_static_pack` is only a stand-in for the device array; its
// device address is looked up once per device, with that device current.
int static_pack_address(double **out) {
  int dev = 0;
  PGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(kErrUnsupported, "device index out of range");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void *p = nullptr;
    PGB_CUDA(cudaGetSymbolAddress(&p, g_static_pack));
    g_static_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_static_ptr[dev];
  return kOk;
}

}  // namespace
}  // namespace pgb

extern "C" int pgb_exchange_static_buffer(pgb_mesh *mesh, double *data, double *coarse, int32_t ncomp,
                                          int32_t flags, void *stream) {
  using namespace pgb;
  GridTables *t = mesh_leaf_tables(mesh);
  if (!t) return fail(kErrState, "mesh is null or its tables are not uploaded (call pgb_mesh_upload)");
  if (ncomp < 1) return fail(kErrInvalid, "ncomp must be positive");
  // the packed-buffer exchange has no sparse form (null buffers are decided per pair
  // by the direct exchange)
  if (mesh_state(mesh)->sparse_dev())
    return fail(kErrUnsupported, "meshes with sparse variables exchange through pgb_exchange without a buffer");
  const size_t need = (size_t)t->buffer_elems * (size_t)ncomp;
  if (need > kStaticPackDoubles)
    return fail(kErrInvalid, "packed exchange needs " + std::to_string(need) +
                                 " doubles, above the static buffer's 4194304 (32 MiB); use pgb_exchange");
  double *buf = nullptr;
  int rc = static_pack_address(&buf);
  if (rc) return rc;
  const int prolongate = flags & PGB_EXCHANGE_PROLONGATE;
  const int op = (flags >> 1) & 3;
  return exchange_grid(*t, data, coarse, ncomp, prolongate, op, buf, (cudaStream_t)stream,
                       mesh_state(mesh)->sparse_dev());
}
