// yc_bdpt.h -- buffers and launchers of the BDPT wavefront (bdpt.cu).
#pragma once

#include <cuda_runtime.h>

#include "yc_internal.h"

namespace yc {

// states of a BDPT path (misc.z & 15)
enum : int {
  // states that wait for a trace result
  B_LIGHT = 0,   // closest hit of the light-subpath ray that makes light vertex i
  B_EYE0 = 1,    // closest hit of the camera ray
  B_EYE = 2,     // closest hit of the eye-subpath ray that makes eye vertex i
  B_NEE = 3,     // shadow ray of the next-event estimate at eye vertex i
  B_CONN = 4,    // connection ray between eye vertex i and light vertex j
  // transient phases
  Q_LIGHT_SAMPLE = 8,
  Q_EYE_START = 9,
  Q_EYE_SAMPLE = 10,
  Q_VERTEX = 11,
  Q_CONNECT = 12,
  Q_FINISH = 13
};

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
                       RoundCounters* rc_out, DevStats* st, int grid, cudaStream_t s, const int* sorted = nullptr,
                       const SortCtl* sctl = nullptr);
// the bidirectional tracer with multiple importance sampling (bdpt_mis.cu): same buffers,
// same trace-state numbering (B_LIGHT .. B_CONN), light vertices only
void launch_raygen_bdpt_mis(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, int* q_closest,
                            RoundCounters* rc, DevStats* st, cudaStream_t s);
void launch_logic_bdpt_mis(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, const int* in_closest,
                           const int* in_any, const RoundCounters* rc_in, int* out_closest, int* out_any,
                           RoundCounters* rc_out, DevStats* st, int grid, cudaStream_t s, const int* sorted = nullptr,
                           const SortCtl* sctl = nullptr);

}  // namespace yc
