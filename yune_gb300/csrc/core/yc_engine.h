// yc_engine.h -- device structures of the batch/serving engine (engine.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "yc_internal.h"

namespace yc {

// One render job: a scene, camera, accumulator and pass list. pp.rand_seed and pp.reset
// are unused (the pass seed comes from `seeds`, the reset flag from reset_first).
struct BatchJob {
  PassParams pp;
  const uint32_t* seeds;   // n_pass per-pass seeds (device)
  int n_pass;
  int reset_first;
  long long task_base;     // first global pixel-task index of this job
  int n_pix;
  int cancelled;           // set between launches: pixels stop after their current pass,
                           // tasks taken in the logic kernel are counted done without work
};

// The task cursor and job count, shared by every slot group of a batch.
struct BatchTasks {
  unsigned long long task_next;    // next unassigned pixel task
  unsigned long long task_total;   // tasks admitted so far
  int n_jobs;
  int pad_;
};

// Control block of one slot group: its free stack and its current fill.
struct BatchCtl {
  int free_top;                    // slots on the group's free stack
  int fill_n;                      // the current fill: tasks claimed for free slots,
  int fill_top;                    //   the free-stack position they are taken from,
  int pad_;
  unsigned long long fill_t0;      //   and the first of them
};

void launch_batch_sort(const BatchJob* jobs, SF<int4> job_pass, const PathState& ps, const int* in_closest,
                       const int* in_any, const RoundCounters* rc_in, int* keys, int* sorted, SortCtl* sctl,
                       int threshold, int grid, cudaStream_t s);

// The ray-sort keys of the rays a kernel queues (RaySortBufs: keys of the closest-hit
// queue, keys of the any-hit queue, the histogram), formed where the rays are written;
// keys_c == nullptr: the rounds are not sorted
struct RsProduce {
  unsigned* keys_c;
  unsigned* keys_a;
  unsigned* hist;
  int ob, db, jb;
};
void launch_batch_fill(const BatchJob* jobs, BatchTasks* tasks, BatchCtl* ctl, const PathState& ps, SF<int4> job_pass,
                       int* free_stack, int* q_closest, RoundCounters* rc, DevStats* st, const RsProduce& rsp, int grid,
                       cudaStream_t s);
void launch_batch_logic(const BatchJob* jobs, BatchTasks* tasks, BatchCtl* ctl, const PathState& ps, SF<int4> job_pass,
                        int* free_stack, const int* in_closest, const int* in_any, const RoundCounters* rc_in,
                        int* out_closest, int* out_any, RoundCounters* rc_out, DevStats* st,
                        unsigned long long* job_done, const int* sorted, const SortCtl* sctl, const RsProduce& rsp,
                        int grid, cudaStream_t s);
// tb: threads per block of the trace kernels (32..256, a multiple of 32)
// The walk stack holds stack_cap entries: n_smem (<= stack_cap) in shared memory, the rest
// in `spill`, one column per thread of the launch (grid_blocks * tb columns of
// 2 * (stack_cap - n_smem) ints; may be null when n_smem == stack_cap).
int launch_batch_trace(bool any_hit, bool wide, const BatchJob* jobs, SF<int4> job_pass, const int* queue,
                       const int* count, int* work, SF<float4> ro, SF<float4> rd, SF<float4> hit, DevStats* st,
                       int stack_cap, int n_smem, int* spill, int grid_blocks, int tb, cudaStream_t s);
int batch_trace_grid(bool any_hit, int n_smem, bool wide, int tb);
// one launch over both queues of a round (closest-hit entries, then any-hit); the work
// cursor is rc->work_closest
int launch_batch_trace_mixed(bool wide, const BatchJob* jobs, SF<int4> job_pass, const int* q_closest,
                             const int* q_any, RoundCounters* rc, SF<float4> ro, SF<float4> rd, SF<float4> hit,
                             DevStats* st, int stack_cap, int n_smem, int* spill, int grid_blocks, int tb,
                             cudaStream_t s, const int* sorted = nullptr, const RaySortCtl* rs = nullptr);
// the same shade-queue sort for the per-pass path (one scene)
void launch_pass_sort(const DevScene& sc, bool bdpt, const PathState& ps, const int* in_closest, const int* in_any,
                      const RoundCounters* rc_in, int* keys, int* sorted, SortCtl* sctl, int threshold, int grid,
                      cudaStream_t s);
// raysort.cu, with the scene box of each ray's job
int launch_raysort_batch(const BatchJob* jobs, SF<int4> job_pass, const int* q_closest, const int* q_any,
                         const RoundCounters* rc, SF<float4> ro, SF<float4> rd, const RaySortBufs& b, int grid,
                         cudaStream_t s);
int batch_trace_mixed_grid(int n_smem, bool wide, int tb);

}  // namespace yc
