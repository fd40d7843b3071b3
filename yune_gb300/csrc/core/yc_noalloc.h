// yc_noalloc.h -- the allocation-free tile render (noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "yc_internal.h"

namespace yc {

// Largest tile (pixels) the static render scratch holds: 16384 paths, about 3.9 MB.
constexpr int NOALLOC_MAX_PATHS = 16384;

struct NoallocPass {
  PassParams pp;
  cudaStream_t stream;
  DevStats* stats;
  RoundCounters* rc_host;   // pinned, owned by the context
  int logic_grid;
  int max_rounds;           // rounds the pass may take (YC_OPT_MAX_ROUNDS)
};

// Runs one pass of the tile described by pp with the static scratch, on the current
// device; returns YC_OK or a YC_E_* code with a message (YC_E_TIMEOUT when paths are still
// live after max_rounds rounds).
int noalloc_render(const NoallocPass& a, std::string& err);

}  // namespace yc
