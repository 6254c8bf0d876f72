// Launch-shape autotuner (see tune.hpp).
#include "tune.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"

namespace pgb {
namespace {

struct Entry {
  int choice = 0;
  std::vector<float> ms;
};

std::mutex g_mu;
std::map<std::string, Entry> g_cache;

}  // namespace

thread_local int g_tune_force = -1;

bool tuning_enabled() {
  const char *e = std::getenv("PGB_TUNE");
  return !(e && e[0] == '0');
}

int tuned_choice(const std::string &key, int fallback) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_cache.find(key);
  return it == g_cache.end() ? fallback : it->second.choice;
}

int tune(const std::string &key, int ncand, int fallback, int reps, const std::function<int(int)> &launch,
         cudaStream_t s) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) return it->second.choice;
  }
  if (!tuning_enabled() || ncand <= 1) return fallback;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return fallback;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fallback;
  }
  Entry en;
  en.ms.assign(ncand, 0.0f);
  bool ok = true;
  for (int c = 0; c < ncand && ok; ++c) {
    if (launch(c) != kOk) {
      ok = false;
      break;
    }
    std::vector<float> t;
    for (int r = 0; r < std::max(1, reps); ++r) {
      cudaEventRecord(e0, s);
      if (launch(c) != kOk) {
        ok = false;
        break;
      }
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        ok = false;
        break;
      }
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      t.push_back(ms);
    }
    if (!ok) break;
    std::sort(t.begin(), t.end());
    en.ms[c] = t[t.size() / 2];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok) return fallback;
  en.choice = (int)(std::min_element(en.ms.begin(), en.ms.end()) - en.ms.begin());
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache[key] = en;
  return en.choice;
}

std::string tune_report() {
  std::lock_guard<std::mutex> lk(g_mu);
  std::string out;
  char buf[64];
  for (auto &kv : g_cache) {
    if (!out.empty()) out += " ; ";
    out += kv.first + "=" + std::to_string(kv.second.choice) + " (";
    for (size_t c = 0; c < kv.second.ms.size(); ++c) {
      std::snprintf(buf, sizeof(buf), "%s%.3f", c ? " " : "", kv.second.ms[c]);
      out += buf;
    }
    out += " ms)";
  }
  return out;
}

}  // namespace pgb

extern "C" int pgb_tune_report(char *buf, int32_t capacity) {
  if (!buf || capacity < 1) return pgb::fail(pgb::kErrInvalid, "null buffer");
  const std::string r = pgb::tune_report();
  const size_t n = std::min<size_t>(r.size(), (size_t)capacity - 1);
  std::copy(r.begin(), r.begin() + n, buf);
  buf[n] = '\0';
  return pgb::kOk;
}
