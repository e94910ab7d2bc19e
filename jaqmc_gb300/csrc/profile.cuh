// Launch counting and per-class event timing (qmc_profile_*).
#pragma once
#include "common.cuh"

namespace qmc {

// RAII bracket around the launches of one kernel class on stream `s`.
struct ProfScope {
  int cls;
  cudaStream_t s;
  int slot;
  ProfScope(int cls, cudaStream_t s);
  ~ProfScope();
};

}  // namespace qmc
