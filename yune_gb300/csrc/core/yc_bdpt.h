// yc_bdpt.h -- buffers and launchers of the BDPT wavefront (bdpt.cu).
#pragma once

#include <cuda_runtime.h>

#include "yc_internal.h"

namespace yc {

// subpath vertices, one 64-byte record (4 float4 fields) per vertex: vertex k of path p,
// field f at [(p * bounces + k) * 4 + f]; `bounces` vertices per subpath (BDPT_BOUNCES)
struct BdptBuffers {
  float4* lv;
  float4* ev;
  size_t N;
  int bounces;
};

void launch_raygen_bdpt(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, int* q_closest,
                        RoundCounters* rc, DevStats* st, cudaStream_t s);
void launch_logic_bdpt(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, const int* in_closest,
                       const int* in_any, const RoundCounters* rc_in, int* out_closest, int* out_any,
                       RoundCounters* rc_out, DevStats* st, int grid, cudaStream_t s);

}  // namespace yc
