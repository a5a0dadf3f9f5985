// tuner.h — autotuner and its on-disk cache.
//
// The reference fixes its schedule at radix 16 (defaultBGl2 = 4,
// FFT_OpenCL_Contiguous.h:55) and one kernel per pass.  Here the plan
// parameters (single kernel vs four-step, N1 x N2 split, elements per thread,
// transforms/columns per CTA, chunk size) are timed on the device and the
// fastest is cached per (GPU, n, log2 batch) in a JSON-lines file:
//   $ESTL_TUNE_CACHE, else $HOME/.cache/estl_gb300/tune.jsonl
#pragma once
#include "planner.h"

namespace estl {

void tuner_load_cache();
bool tuner_lookup(long long n, long long batch, PlanChoice* out);
void tuner_store(long long n, long long batch, const PlanChoice& c, double ms);
std::string tuner_cache_path();
std::string choice_to_json(const PlanChoice& c);

}  // namespace estl
