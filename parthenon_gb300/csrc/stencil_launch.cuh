// Host launchers for one stencil build (included once by stencil_exact.cu and once by
// stencil_fast.cu after stencil_impl.cuh).
#pragma once

namespace pgb {
namespace PGB_NS {

template <int NC, bool BURGERS>
int launch_stage_nc(const StageArgs &a, bool store_flux, cudaStream_t s) {
  const Dims &d = a.d;
  auto grid_for = [&](int D) {
    const int64_t nf = D == 0 ? d.nx[1] : d.nx[0];
    const int64_t ns = D == 2 ? d.nx[1] : d.nx[2];
    const int64_t lines = (int64_t)a.nblocks * nf * ns;
    return dim3((unsigned)((lines + 127) / 128));
  };
  if (BURGERS) {
    if (store_flux) {
      k_march<NC, 0, kStoreFlux><<<grid_for(0), 128, 0, s>>>(a);
      k_march<NC, 1, kStoreFlux><<<grid_for(1), 128, 0, s>>>(a);
      k_march<NC, 2, kStoreFlux><<<grid_for(2), 128, 0, s>>>(a);
    } else {
      k_march<NC, 0, kStoreDu><<<grid_for(0), 128, 0, s>>>(a);
      k_march<NC, 1, kAddDu><<<grid_for(1), 128, 0, s>>>(a);
      k_march<NC, 2, kFinishUpdate><<<grid_for(2), 128, 0, s>>>(a);
    }
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrCuda;
}

// Advection: one component per thread (grid.y = component), any component count.
int launch_advection(const StageArgs &a, bool store_flux, cudaStream_t s) {
  const Dims &d = a.d;
  auto g = [&](int D) {
    const int64_t nf = D == 0 ? d.nx[1] : d.nx[0];
    const int64_t ns = D == 2 ? d.nx[1] : d.nx[2];
    const int64_t lines = (int64_t)a.nblocks * nf * ns;
    return dim3((unsigned)((lines + 127) / 128), (unsigned)a.ncomp);
  };
#ifdef PGB_HAVE_PLM_X_STAGED
  // fast build, PLM: the x sweep from lines staged in shared memory (advection_df.cuh)
  const bool staged = a.recon != 0 && d.nx[0] <= kXStageMaxN;
#else
  const bool staged = false;
#endif
  if (store_flux) {
#ifdef PGB_HAVE_PLM_X_STAGED
    if (staged) k_march_adv_x_df<kStoreFlux><<<g(0), 128, x_stage_smem(d.nx[0]), s>>>(a);
#endif
    if (!staged) k_march_adv<0, kStoreFlux><<<g(0), 128, 0, s>>>(a);
    k_march_adv<1, kStoreFlux><<<g(1), 128, 0, s>>>(a);
    k_march_adv<2, kStoreFlux><<<g(2), 128, 0, s>>>(a);
  } else {
#ifdef PGB_HAVE_PLM_X_STAGED
    if (staged) k_march_adv_x_df<kStoreDu><<<g(0), 128, x_stage_smem(d.nx[0]), s>>>(a);
#endif
    if (!staged) k_march_adv<0, kStoreDu><<<g(0), 128, 0, s>>>(a);
    k_march_adv<1, kAddDu><<<g(1), 128, 0, s>>>(a);
    k_march_adv<2, kFinishUpdate><<<g(2), 128, 0, s>>>(a);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrCuda;
}

template <int NC>
int launch_div_update_nc(const StageArgs &a, cudaStream_t s) {
  const int64_t cells = (int64_t)a.nblocks * a.d.nx[0] * a.d.nx[1] * a.d.nx[2];
  k_div_update<NC><<<(unsigned)((cells + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrCuda;
}

// physics 0 = advection, 1 = Burgers; store_flux selects the multilevel path.
int launch_stage(const StageArgs &a, int ncomp, int physics, bool store_flux, cudaStream_t s) {
#ifdef PGB_HAVE_BURGERS_FAST
  // WENO5: per-face HLL coefficients shared by all components (uniform and multilevel)
  if (physics == 1 && a.recon == 0) {
    switch (ncomp) {
      case 4: return launch_burgers_nc<4>(a, store_flux, s);
      case 5: return launch_burgers_nc<5>(a, store_flux, s);
      case 11: return launch_burgers_nc<11>(a, store_flux, s);
      default: break;
    }
  }
#endif
  if (physics == 1) {
    switch (ncomp) {
      case 4: return launch_stage_nc<4, true>(a, store_flux, s);
      case 5: return launch_stage_nc<5, true>(a, store_flux, s);
      case 11: return launch_stage_nc<11, true>(a, store_flux, s);
      default: return kErrUnsupported;
    }
  }
  if (ncomp < 1 || ncomp > 65535) return kErrUnsupported;
  return launch_advection(a, store_flux, s);
}

int launch_div_update(const StageArgs &a, int ncomp, cudaStream_t s) {
  switch (ncomp) {
    case 1: return launch_div_update_nc<1>(a, s);
    case 4: return launch_div_update_nc<4>(a, s);
    case 5: return launch_div_update_nc<5>(a, s);
    case 11: return launch_div_update_nc<11>(a, s);
    default: return ncomp >= 1 ? launch_div_update_nc<0>(a, s) : kErrUnsupported;
  }
}

}  // namespace PGB_NS
}  // namespace pgb
