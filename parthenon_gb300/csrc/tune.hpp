// Launch-shape autotuner.
//
// Some launch parameters have no single best value across meshes (threads per CTA of
// the ghost copy, persistent CTAs per SM of the WENO5/HLL sweep). For each kernel
// family and problem signature the tuner times a few candidate shapes on the caller's
// own data with CUDA events, once, outside any graph capture, and caches the fastest
// for the process; launches then read the cached choice (or a fixed default when
// nothing was tuned). Tuning is off when the environment sets PGB_TUNE=0.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>

namespace pgb {

// Cached choice for `key`, or `fallback` when the key was never tuned.
int tuned_choice(const std::string &key, int fallback);
// Times launch(c) for c in [0, ncand) on stream s (one untimed run, then `reps` timed
// runs; the median counts) and caches the fastest. launch must be idempotent and must
// not be under stream capture. Returns the chosen index (fallback when tuning is off).
int tune(const std::string &key, int ncand, int fallback, int reps, const std::function<int(int)> &launch,
         cudaStream_t s);
bool tuning_enabled();
// "key=choice (ms per candidate) ; ..." for reports
std::string tune_report();

// Candidate under test while a tuner runs a launch (-1 otherwise); the launch code
// reads it before the cache.
extern thread_local int g_tune_force;

// Persistent CTAs per SM of the WENO5/HLL directional sweep.
constexpr int kBurgersGridMult[4] = {1, 2, 4, 8};
constexpr int kBurgersGridCandidates = 4;
constexpr int kBurgersGridDefault = 1;  // index: 2 CTAs per SM
// Threads per CTA of the direct ghost copy.
constexpr int kCopyThreads[3] = {64, 128, 256};
constexpr int kCopyThreadsDefault = 1;  // index: 128

inline std::string burgers_tune_key(int nc, int n, bool flux, int nblocks) {
  int b = 0;
  while ((1 << (b + 1)) <= nblocks) ++b;  // blocks bucketed by powers of two
  return "burgers_dir nc=" + std::to_string(nc) + " n=" + std::to_string(n) + (flux ? " flux" : " du") +
         " blocks~2^" + std::to_string(b);
}
inline std::string copy_tune_key(int ncomp, int npairs, int n) {
  int b = 0;
  while ((1 << (b + 1)) <= npairs) ++b;
  return "k_copy ncomp=" + std::to_string(ncomp) + " n=" + std::to_string(n) + " pairs~2^" + std::to_string(b);
}

}  // namespace pgb
