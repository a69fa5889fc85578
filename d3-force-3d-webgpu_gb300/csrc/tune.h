// The autotuner behind fl_autotune and fl_batch_autotune (host code).
//
// A coordinate descent over tuning knobs: each knob in turn takes each of its candidate values
// with the others held at their best so far, and keeps the fastest (a candidate must beat the
// current best by more than kTuneMargin, so timing noise does not flip a choice). The caller
// supplies how to set a knob and how to time a configuration. Results are cached per
// configuration key in a text file, one line per key:
//   <key>\t<knob>=<value> ... ms=<best> default_ms=<defaults>
// A key found in the file is applied without timing anything.
#pragma once

#include <functional>
#include <string>
#include <vector>

struct FlTuneKnob {
  int key;                 // FL_TUNE_*
  const char* name;        // its name in the cache file
  std::vector<int> values; // candidates; the first is the default
  int chosen;              // out: the value kept
};

struct FlTuneOutcome {
  double best_ms = 0, default_ms = 0;
  int candidates = 0;  // configurations timed
  bool cached = false;
};

// Returns 0, or the first nonzero code that set() or time() returned (the knobs are then left as
// set() last set them). time() returns the ms per tick of the current configuration in *ms.
int fl_tune_search(const char* cache_path, const std::string& cache_key,
                   std::vector<FlTuneKnob>& knobs, const std::function<int(int, int)>& set,
                   const std::function<int(double*)>& time, FlTuneOutcome* out);

// The compute capability as "sm<major><minor>" for cache keys.
std::string fl_tune_arch();
