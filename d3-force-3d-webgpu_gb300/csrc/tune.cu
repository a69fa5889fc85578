// The autotuner's search and cache (declared in tune.h).
#include "tune.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

namespace {

constexpr double kTuneMargin = 0.01;  // a candidate must be 1 % faster to replace the best

// The cached values of `key`, if the file holds a line for it.
bool read_cache(const char* path, const std::string& key, std::vector<FlTuneKnob>& knobs,
                FlTuneOutcome* out) {
  if (!path || !*path) return false;
  std::ifstream f(path);
  if (!f) return false;
  std::string line;
  while (std::getline(f, line)) {
    const size_t tab = line.find('\t');
    if (tab == std::string::npos || line.compare(0, tab, key) != 0 || tab != key.size()) continue;
    std::istringstream rest(line.substr(tab + 1));
    std::string item;
    std::vector<int> got(knobs.size(), 0);
    std::vector<bool> seen(knobs.size(), false);
    double ms = 0, dms = 0;
    while (rest >> item) {
      const size_t eq = item.find('=');
      if (eq == std::string::npos) continue;
      const std::string name = item.substr(0, eq), val = item.substr(eq + 1);
      if (name == "ms") ms = std::atof(val.c_str());
      else if (name == "default_ms") dms = std::atof(val.c_str());
      for (size_t k = 0; k < knobs.size(); ++k)
        if (name == knobs[k].name) got[k] = std::atoi(val.c_str()), seen[k] = true;
    }
    bool all = true;
    for (size_t k = 0; k < knobs.size(); ++k) all = all && seen[k];
    if (!all) continue;  // a line from a build with other knobs: time afresh
    for (size_t k = 0; k < knobs.size(); ++k) knobs[k].chosen = got[k];
    out->best_ms = ms, out->default_ms = dms, out->cached = true;
    return true;
  }
  return false;
}

void write_cache(const char* path, const std::string& key, const std::vector<FlTuneKnob>& knobs,
                 const FlTuneOutcome& o) {
  if (!path || !*path) return;
  std::ofstream f(path, std::ios::app);
  if (!f) return;  // an unwritable cache only costs the next run a search
  f << key << '\t';
  for (auto& k : knobs) f << k.name << '=' << k.chosen << ' ';
  char buf[96];
  std::snprintf(buf, sizeof buf, "ms=%.5f default_ms=%.5f", o.best_ms, o.default_ms);
  f << buf << '\n';
}

}  // namespace

std::string fl_tune_arch() {
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return "sm" + std::to_string(major) + std::to_string(minor);
}

int fl_tune_search(const char* cache_path, const std::string& cache_key,
                   std::vector<FlTuneKnob>& knobs, const std::function<int(int, int)>& set,
                   const std::function<int(double*)>& time, FlTuneOutcome* out) {
  *out = FlTuneOutcome{};
  int rc;
  if (read_cache(cache_path, cache_key, knobs, out)) {
    for (auto& k : knobs)
      if ((rc = set(k.key, k.chosen)) != 0) return rc;
    return 0;
  }
  for (auto& k : knobs) {
    k.chosen = k.values.empty() ? 0 : k.values[0];
    if ((rc = set(k.key, k.chosen)) != 0) return rc;
  }
  double best = 0;
  if ((rc = time(&best)) != 0) return rc;
  out->default_ms = best;
  out->candidates = 1;
  for (auto& k : knobs) {
    for (size_t i = 1; i < k.values.size(); ++i) {
      if ((rc = set(k.key, k.values[i])) != 0) return rc;
      double ms = 0;
      if ((rc = time(&ms)) != 0) return rc;
      ++out->candidates;
      if (ms < best * (1.0 - kTuneMargin)) best = ms, k.chosen = k.values[i];
    }
    if ((rc = set(k.key, k.chosen)) != 0) return rc;
  }
  out->best_ms = best;
  write_cache(cache_path, cache_key, knobs, *out);
  return 0;
}
