// engine.cu -- batch and serving engine: many render jobs in one persistent wavefront.
//
// A batch owns a fixed pool of path slots. Every job (scene, camera, accumulator, pass
// seeds) contributes one pixel task per pixel; a slot takes a task, renders that pixel's
// passes one after the other (each pass is a full `pathtracer` sample, udpt.cl:158-211,
// accumulated in pass order, so every pixel's result is bit-identical to the per-pass
// path), then takes the next task. Slots regenerate in place inside the logic kernel
// (path regeneration), so the wavefront stays full while jobs of any size and
// resolution start and finish; the extend and occlusion kernels read each ray's scene
// from the job table, so one launch walks many BVHs. Jobs can be added between launches
// (serving); a task claim is one atomicAdd on the task cursor, and a job added later
// starts at or after the cursor, so its tasks are never skipped. The pool is split into
// slot groups, each with its own free stack and queues, whose rounds run concurrently
// on their own streams and take tasks from the one shared cursor: while one group's
// round waits on its last rays, the other groups' kernels use the idle SMs.
#include <cuda_runtime.h>

#include "yc_bdpt.h"
#include "yc_engine.h"
#include "yc_trace_loop.cuh"
#include "yc_udpt.cuh"

namespace yc {

constexpr int ENGINE_TB = 256;

__device__ __forceinline__ int job_of_task(const BatchJob* jobs, int n_jobs, unsigned long long t) {
  int lo = 0, hi = n_jobs - 1;
  while (lo < hi) {   // last job with task_base <= t
    const int mid = (lo + hi + 1) >> 1;
    if ((unsigned long long)jobs[mid].task_base <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// first pass (or the next pass) of pixel `pix` of job `job` in slot p
__device__ __forceinline__ void start_pass(const BatchJob& J, int job, int pix, int pass, int p, const PathState& ps,
                                           SF<int4> job_pass) {
  const int W = J.pp.width;
  uint32_t seed;
  f4 o, d;
  float len;
  int k;
  camera_ray(J.pp, pix % W, pix / W, J.seeds[pass], seed, o, d, len, k);
  ps.misc[p] = make_int4((int)seed, pix, pack_misc(S_PRIMARY, 0, -1, k), 0);
  ps.ro[p] = make_float4(o.x, o.y, o.z, len);
  ps.rd[p] = make_float4(d.x, d.y, d.z, d.w);
  job_pass[p] = make_int4(job, pass, 0, 0);
}

// Claims up to `want` consecutive tasks below task_total; returns the first and sets got.
// One atomicAdd per claim: the cursor may run past task_total (those tasks do not exist
// and are dropped); yc_batch_add_job starts a new job at or after the cursor, so no task
// admitted later falls into the overshoot.
__device__ __forceinline__ unsigned long long claim_tasks(BatchTasks* tasks, int want, int& got) {
  const unsigned long long total = *(volatile unsigned long long*)&tasks->task_total;
  if (*(volatile unsigned long long*)&tasks->task_next >= total) { got = 0; return total; }
  const unsigned long long t = atomicAdd(&tasks->task_next, (unsigned long long)want);
  got = t >= total ? 0 : (int)((total - t) < (unsigned long long)want ? (total - t) : (unsigned long long)want);
  return t;
}

// ---- ray-sort keys formed by the kernels that queue the rays ----
// The queued ray of slot p (ps.ro / ps.rd as just written, the scene box of its job) gets
// the key of k_rs_key (raysort.cu) at its queue position; the warp's equal keys are
// counted with one histogram atomic. Every lane of the warp calls it (kind 0: no ray).
__device__ __forceinline__ void produce_key(const RsProduce& rsp, const BatchJob* jobs, const PathState& ps,
                                            SF<int4> job_pass, int p, int kind, int pos) {
  const int lane = threadIdx.x & 31;
  unsigned key = 0xffffffffu - lane;   // lanes without a ray match nobody
  if (kind) {
    const float4 o = ps.ro[p], d = ps.rd[p];
    const unsigned job = (unsigned)job_pass[p].x;
    const DevScene& sc = jobs[job].pp.sc;
    key = ray_key(o, d, sc.root_lo, sc.root_hi, rsp.ob, rsp.db) |
          ((job & ((1u << rsp.jb) - 1u)) << (3 * (rsp.ob + rsp.db))) |
          (kind == 2 ? 1u << (3 * (rsp.ob + rsp.db) + rsp.jb) : 0u);
    (kind == 1 ? rsp.keys_c : rsp.keys_a)[pos] = key;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  if (kind && lane == __ffs(peers) - 1) atomicAdd(&rsp.hist[key], (unsigned)__popc(peers));
}

// ---- fill: idle slots (on the free stack) take new tasks ----
// k_batch_plan claims, in one thread, as many tasks as there are free slots; k_batch_fill
// then starts them across the grid.
__global__ void k_batch_plan(BatchTasks* tasks, BatchCtl* ctl) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int free_n = ctl->free_top;
  int got = 0;
  const unsigned long long t0 = free_n > 0 ? claim_tasks(tasks, free_n, got) : 0ull;
  ctl->fill_t0 = t0;
  ctl->fill_n = got;
  ctl->fill_top = free_n - got;
  ctl->free_top = free_n - got;
}

__global__ void __launch_bounds__(ENGINE_TB) k_batch_fill(const BatchJob* __restrict__ jobs,
                                                          const BatchTasks* tasks, const BatchCtl* ctl,
                                                          PathState ps, SF<int4> job_pass, const int* free_stack,
                                                          int* q_closest, RoundCounters* rc, DevStats* st,
                                                          RsProduce rsp) {
  const int n = ctl->fill_n;
  const int top = ctl->fill_top;
  const unsigned long long t0 = ctl->fill_t0;
  const int n_jobs = tasks->n_jobs;
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  unsigned long long started = 0;
  for (int wbase = warp_global * 32; wbase < n; wbase += warps_total * 32) {
    const int i = wbase + lane;
    const bool active = i < n;
    int p = -1;
    if (active) {
      p = free_stack[top + i];
      const unsigned long long t = t0 + (unsigned long long)i;
      const int job = job_of_task(jobs, n_jobs, t);
      start_pass(jobs[job], job, (int)(t - (unsigned long long)jobs[job].task_base), 0, p, ps, job_pass);
    }
    const unsigned m = __ballot_sync(0xffffffffu, active);
    int b = 0;
    if (lane == 0) b = atomicAdd(&rc->n_closest, __popc(m));
    b = __shfl_sync(0xffffffffu, b, 0);
    const int pos = b + __popc(m & ((1u << lane) - 1));
    if (active) q_closest[pos] = p;
    if (rsp.keys_c) produce_key(rsp, jobs, ps, job_pass, p, active ? 1 : 0, pos);
    started += __popc(m);
  }
  if (lane == 0 && started) {
    atomicAdd(&st->primary, started);
    atomicAdd(&st->rays, started);
    atomicAdd(&st->traversed, started);
  }
}

void launch_batch_fill(const BatchJob* jobs, BatchTasks* tasks, BatchCtl* ctl, const PathState& ps, SF<int4> job_pass,
                       int* free_stack, int* q_closest, RoundCounters* rc, DevStats* st, const RsProduce& rsp, int grid,
                       cudaStream_t s) {
  k_batch_plan<<<1, 32, 0, s>>>(tasks, ctl);
  k_batch_fill<<<grid, ENGINE_TB, 0, s>>>(jobs, tasks, ctl, ps, job_pass, free_stack, q_closest, rc, st, rsp);
}

// ---- logic with regeneration ----
__global__ void __launch_bounds__(ENGINE_TB) k_batch_logic(const BatchJob* __restrict__ jobs, BatchTasks* tasks,
                                                           BatchCtl* ctl,
                                                           PathState ps, SF<int4> job_pass, int* free_stack,
                                                           const int* __restrict__ in_closest,
                                                           const int* __restrict__ in_any, const RoundCounters* rc_in,
                                                           int* out_closest, int* out_any, RoundCounters* rc_out,
                                                           DevStats* st, unsigned long long* job_done,
                                                           const int* __restrict__ sorted, const SortCtl* sctl,
                                                           RsProduce rsp) {
  __shared__ unsigned long long s_cnt[8];
  if (threadIdx.x < 8) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const int nc = rc_in->n_closest, na = rc_in->n_any;
  const int n = nc + na;
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const int n_jobs = tasks->n_jobs;
  const bool use_sorted = sctl->use != 0;
  for (int wbase = warp_global * 32; wbase < n; wbase += warps_total * 32) {
    const int e = wbase + lane;
    int emit = 0;
    int p = -1;
    bool need_task = false;
    LogicCounts lc;
    if (e < n) {
      p = use_sorted ? sorted[e] : (e < nc ? in_closest[e] : in_any[e - nc]);
      const int4 jp = job_pass[p];
      const BatchJob& J = jobs[jp.x];
      const int reset = (jp.y == 0) ? J.reset_first : 0;
      emit = logic_path(J.pp, reset, ps, p, lc);
      if (emit == 0) {
        if (jp.y + 1 < J.n_pass && !J.cancelled) {   // next pass of the same pixel
          start_pass(J, jp.x, ps.misc[p].y, jp.y + 1, p, ps, job_pass);
          emit = 1;
          lc.rays++; lc.trav++; lc.prim++;
        } else {
          atomicAdd(&job_done[jp.x], 1ull);
          need_task = true;
        }
      }
    }
    // slots whose pixel is done take the next tasks, one claim per warp; a task of a
    // cancelled job is counted done without work and the slot claims again (a few times
    // at most: then it waits on the free stack for the next launch's fill)
    for (int attempt = 0; attempt < 4; ++attempt) {
      const unsigned mt = __ballot_sync(0xffffffffu, need_task);
      if (!mt) break;
      unsigned long long t0 = 0;
      int got = 0;
      if (lane == 0) t0 = claim_tasks(tasks, __popc(mt), got);
      t0 = __shfl_sync(0xffffffffu, t0, 0);
      got = __shfl_sync(0xffffffffu, got, 0);
      if (need_task) {
        const int rank = __popc(mt & ((1u << lane) - 1));
        if (rank < got) {
          const unsigned long long t = t0 + (unsigned long long)rank;
          const int job = job_of_task(jobs, n_jobs, t);
          if (jobs[job].cancelled) {
            atomicAdd(&job_done[job], 1ull);
          } else {
            start_pass(jobs[job], job, (int)(t - (unsigned long long)jobs[job].task_base), 0, p, ps, job_pass);
            emit = 1;
            lc.rays++; lc.trav++; lc.prim++;
            need_task = false;
          }
        } else {
          free_stack[atomicAdd(&ctl->free_top, 1)] = p;
          need_task = false;
        }
      }
    }
    if (need_task) free_stack[atomicAdd(&ctl->free_top, 1)] = p;
    const unsigned mc = __ballot_sync(0xffffffffu, emit == 1);
    const unsigned ma = __ballot_sync(0xffffffffu, emit == 2);
    int bc = 0, ba = 0;
    if (lane == 0) {
      if (mc) bc = atomicAdd(&rc_out->n_closest, __popc(mc));
      if (ma) ba = atomicAdd(&rc_out->n_any, __popc(ma));
    }
    bc = __shfl_sync(0xffffffffu, bc, 0);
    ba = __shfl_sync(0xffffffffu, ba, 0);
    const unsigned below = (1u << lane) - 1;
    const int pos = emit == 1 ? bc + __popc(mc & below) : ba + __popc(ma & below);
    if (emit == 1) out_closest[pos] = p;
    if (emit == 2) out_any[pos] = p;
    if (rsp.keys_c) produce_key(rsp, jobs, ps, job_pass, p, emit, pos);
    unsigned v[7] = {lc.rays, lc.ext, lc.shadow, lc.mis, lc.trav, lc.samples, lc.prim};
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      unsigned x = v[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
      if (lane == 0 && x) atomicAdd(&s_cnt[q], (unsigned long long)x);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_cnt[0]) atomicAdd(&st->rays, s_cnt[0]);
    if (s_cnt[1]) atomicAdd(&st->extension, s_cnt[1]);
    if (s_cnt[2]) atomicAdd(&st->shadow, s_cnt[2]);
    if (s_cnt[3]) atomicAdd(&st->mis, s_cnt[3]);
    if (s_cnt[4]) atomicAdd(&st->traversed, s_cnt[4]);
    if (s_cnt[5]) atomicAdd(&st->samples, s_cnt[5]);
    if (s_cnt[6]) atomicAdd(&st->primary, s_cnt[6]);
  }
}

void launch_batch_logic(const BatchJob* jobs, BatchTasks* tasks, BatchCtl* ctl, const PathState& ps, SF<int4> job_pass,
                        int* free_stack,
                        const int* in_closest, const int* in_any, const RoundCounters* rc_in, int* out_closest,
                        int* out_any, RoundCounters* rc_out, DevStats* st, unsigned long long* job_done,
                        const int* sorted, const SortCtl* sctl, const RsProduce& rsp, int grid, cudaStream_t s) {
  k_batch_logic<<<grid, ENGINE_TB, 0, s>>>(jobs, tasks, ctl, ps, job_pass, free_stack, in_closest, in_any, rc_in,
                                           out_closest, out_any, rc_out, st, job_done, sorted, sctl, rsp);
}

// ---- shade-queue sort (counting sort over SORT_KEYS keys) ----
__device__ __forceinline__ int material_class(const yc_material& m) {
  if (m.is_specular) return m.is_transmissive ? 3 : 2;
  return (m.ks.x > 0.0f || m.ks.y > 0.0f || m.ks.z > 0.0f) ? 1 : 0;   // a glossy lobe can be drawn
}

// the scene of the path in slot p: its job's scene in a batch, or the pass's one scene
struct SceneOfBatch {
  const BatchJob* jobs;
  SF<int4> job_pass;
  __device__ __forceinline__ const DevScene& of(int p) const { return jobs[job_pass[p].x].pp.sc; }
};
struct SceneOfOne {
  DevScene sc;
  __device__ __forceinline__ const DevScene& of(int) const { return sc; }
};

// unidirectional paths: the phase, and the material of the surface the step shades
struct KeyUdpt {
  template <class SceneOf>
  __device__ __forceinline__ int operator()(const SceneOf& so, const PathState& ps, int p) const {
    const DevScene& sc = so.of(p);
    const int st = ps.misc[p].z & 15;   // the phase a path waits in: S_PRIMARY..S_EXT
    int mat;
    if (st == S_PRIMARY || st == S_EXT) {
      const int tri = __float_as_int(ps.hit[p].w);
      if (tri < 0) return st * 5 + 4;
      mat = __float_as_int(__ldg(sc.shade + 4 * (size_t)tri + 3).x);
    } else {
      mat = __float_as_int(ps.wi[p].w);
    }
    return st * 5 + material_class(sc.mats[mat]);
  }
};
// BDPT paths: the state, and for a closest-hit result the material of the surface hit
struct KeyBdpt {
  template <class SceneOf>
  __device__ __forceinline__ int operator()(const SceneOf& so, const PathState& ps, int p) const {
    const int st = ps.misc[p].z & 15;   // B_LIGHT..B_CONN
    if (st == B_NEE || st == B_CONN) return st * 5;
    const int tri = __float_as_int(ps.hit[p].w);
    if (tri < 0) return st * 5 + 4;
    const DevScene& sc = so.of(p);
    return st * 5 + material_class(sc.mats[__float_as_int(__ldg(sc.shade + 4 * (size_t)tri + 3).x)]);
  }
};

template <class SceneOf, class Key>
__global__ void __launch_bounds__(ENGINE_TB) k_sort_hist(SceneOf so, Key key_of, PathState ps,
                                                         const int* __restrict__ in_closest,
                                                         const int* __restrict__ in_any, const RoundCounters* rc_in,
                                                         int* keys, SortCtl* sctl, int threshold) {
  __shared__ int h[SORT_KEYS];
  if (threadIdx.x < SORT_KEYS) h[threadIdx.x] = 0;
  __syncthreads();
  const int nc = rc_in->n_closest, n = nc + rc_in->n_any;
  if (n < threshold) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int p = e < nc ? in_closest[e] : in_any[e - nc];
    const int key = key_of(so, ps, p);
    keys[e] = key;
    atomicAdd(&h[key], 1);
  }
  __syncthreads();
  if (threadIdx.x < SORT_KEYS && h[threadIdx.x]) atomicAdd(&sctl->count[threadIdx.x], h[threadIdx.x]);
}

__global__ void k_sort_scan(const RoundCounters* rc_in, SortCtl* sctl, int threshold) {
  if (threadIdx.x != 0) return;
  const int n = rc_in->n_closest + rc_in->n_any;
  const int use = (threshold > 0 && n >= threshold) ? 1 : 0;
  if (use) {
    int run = 0;
    for (int k = 0; k < SORT_KEYS; ++k) {
      sctl->cursor[k] = run;
      run += sctl->count[k];
    }
  }
  sctl->use = use;
}

// Scatter in tiles of SORT_U x 256 entries per block: the tile's entries take their
// offsets within the tile from shared counters (one shared atomic per run of equal keys
// in a warp), then one global atomic per key and tile reserves the tile's range. The
// 25 keys would otherwise put every warp's atomics on the same few addresses.
constexpr int SORT_U = 8;

__global__ void __launch_bounds__(ENGINE_TB) k_sort_scatter(const int* __restrict__ in_closest,
                                                            const int* __restrict__ in_any, const RoundCounters* rc_in,
                                                            const int* __restrict__ keys, int* sorted, SortCtl* sctl) {
  __shared__ int s_cnt[SORT_KEYS];
  __shared__ int s_base[SORT_KEYS];
  if (!sctl->use) return;
  const int nc = rc_in->n_closest, n = nc + rc_in->n_any;
  const int lane = threadIdx.x & 31;
  const int tile = ENGINE_TB * SORT_U;
  // t0 is the same for every thread of the block, so the barriers below are uniform
  for (int t0 = blockIdx.x * tile; t0 < n; t0 += gridDim.x * tile) {
    if (threadIdx.x < SORT_KEYS) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    const int wbase = t0 + (threadIdx.x >> 5) * 32 * SORT_U;
    int key[SORT_U], off[SORT_U], val[SORT_U];
#pragma unroll
    for (int u = 0; u < SORT_U; ++u) {
      const int e = wbase + u * 32 + lane;
      const bool active = e < n;
      key[u] = active ? keys[e] : -1 - lane;   // idle lanes match nobody
      val[u] = active ? (e < nc ? in_closest[e] : in_any[e - nc]) : 0;
    }
#pragma unroll
    for (int u = 0; u < SORT_U; ++u) {
      const int e = wbase + u * 32 + lane;
      const unsigned peers = __match_any_sync(0xffffffffu, key[u]);
      const int leader = __ffs(peers) - 1;
      int b = 0;
      if (e < n && lane == leader) b = atomicAdd(&s_cnt[key[u]], __popc(peers));
      off[u] = __shfl_sync(0xffffffffu, b, leader) + __popc(peers & ((1u << lane) - 1));
    }
    __syncthreads();
    if (threadIdx.x < SORT_KEYS) {
      const int c = s_cnt[threadIdx.x];
      s_base[threadIdx.x] = c ? atomicAdd(&sctl->cursor[threadIdx.x], c) : 0;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < SORT_U; ++u) {
      const int e = wbase + u * 32 + lane;
      if (e < n) sorted[s_base[key[u]] + off[u]] = val[u];
    }
    __syncthreads();   // s_cnt and s_base are reset by the next tile
  }
}

void launch_batch_sort(const BatchJob* jobs, SF<int4> job_pass, const PathState& ps, const int* in_closest,
                       const int* in_any, const RoundCounters* rc_in, int* keys, int* sorted, SortCtl* sctl,
                       int threshold, int grid, cudaStream_t s) {
  k_sort_hist<<<grid, ENGINE_TB, 0, s>>>(SceneOfBatch{jobs, job_pass}, KeyUdpt{}, ps, in_closest, in_any, rc_in, keys,
                                         sctl, threshold);
  k_sort_scan<<<1, 32, 0, s>>>(rc_in, sctl, threshold);
  k_sort_scatter<<<grid, ENGINE_TB, 0, s>>>(in_closest, in_any, rc_in, keys, sorted, sctl);
}

void launch_pass_sort(const DevScene& sc, bool bdpt, const PathState& ps, const int* in_closest, const int* in_any,
                      const RoundCounters* rc_in, int* keys, int* sorted, SortCtl* sctl, int threshold, int grid,
                      cudaStream_t s) {
  if (bdpt)
    k_sort_hist<<<grid, ENGINE_TB, 0, s>>>(SceneOfOne{sc}, KeyBdpt{}, ps, in_closest, in_any, rc_in, keys, sctl,
                                           threshold);
  else
    k_sort_hist<<<grid, ENGINE_TB, 0, s>>>(SceneOfOne{sc}, KeyUdpt{}, ps, in_closest, in_any, rc_in, keys, sctl,
                                           threshold);
  k_sort_scan<<<1, 32, 0, s>>>(rc_in, sctl, threshold);
  k_sort_scatter<<<grid, ENGINE_TB, 0, s>>>(in_closest, in_any, rc_in, keys, sorted, sctl);
}

// ---- traversal with a scene per ray ----
template <bool ANY>
struct BatchSrc {
  const BatchJob* jobs;
  SF<int4> job_pass;
  const int* __restrict__ queue;
  SF<float4> ro;
  SF<float4> rd;
  SF<float4> hit;
  __device__ __forceinline__ const DevScene& begin(int e, RayIn& r) {
    const int q = queue[e];
    const float4 o = __ldg(&ro[q]);
    const float4 d = __ldg(&rd[q]);
    r = RayIn{o.x, o.y, o.z, o.w, d.x, d.y, d.z};
    return jobs[job_pass[q].x].pp.sc;
  }
  __device__ __forceinline__ void end(int e, const HitOut& h) {
    const int q = queue[e];
    if (ANY) hit[q] = make_float4(h.tri >= 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
    else hit[q] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
  }
};

template <bool ANY, bool WIDE>
__global__ void __launch_bounds__(TRACE_TB_MAX) k_batch_trace(const BatchJob* jobs, SF<int4> job_pass,
                                                          const int* __restrict__ queue, const int* __restrict__ count,
                                                          int* work, SF<float4> ro,
                                                          SF<float4> rd, SF<float4> hit, int stack_cap,
                                                          DevStats* st, int n_smem, int* spill) {
  BatchSrc<ANY> src{jobs, job_pass, queue, ro, rd, hit};
  trace_loop<ANY, WIDE>(src, *count, work, stack_cap, st, n_smem, spill);
}

// both queues of a round: closest-hit entries first, then any-hit (or the sorted list,
// which keeps that split)
struct BatchMixedSrc {
  const BatchJob* jobs;
  SF<int4> job_pass;
  const int* __restrict__ q_closest;
  const int* __restrict__ q_any;
  const int* __restrict__ sorted;   // non-null: this round's sorted work list
  int nc;
  SF<float4> ro;
  SF<float4> rd;
  SF<float4> hit;
  __device__ __forceinline__ int slot(int e, bool any) const {
    return sorted ? sorted[e] : (any ? q_any[e - nc] : q_closest[e]);
  }
  __device__ __forceinline__ const DevScene& begin(int e, bool any, RayIn& r) {
    const int q = slot(e, any);
    const float4 o = __ldg(&ro[q]);
    const float4 d = __ldg(&rd[q]);
    r = RayIn{o.x, o.y, o.z, o.w, d.x, d.y, d.z};
    return jobs[job_pass[q].x].pp.sc;
  }
  __device__ __forceinline__ void end(int e, bool any, const HitOut& h) {
    const int q = slot(e, any);
    hit[q] = any ? make_float4(h.tri >= 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f)
                 : make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
  }
};

// At most 64 registers a thread (four blocks of 256 or eight of 128 threads per SM): with
// the walk stack mostly outside shared memory (stack_smem) the traversal is bound by the
// latency of its node and triangle fetches, and the extra warps hide more of it than the
// few spilled registers cost (measured on the mixed workload: +4% over 78 registers).
template <bool WIDE>
__global__ void __launch_bounds__(TRACE_TB_MAX, 4) k_batch_trace_mixed(const BatchJob* jobs, SF<int4> job_pass,
                                                                const int* __restrict__ q_closest,
                                                                const int* __restrict__ q_any,
                                                                RoundCounters* rc, SF<float4> ro,
                                                                SF<float4> rd, SF<float4> hit,
                                                                int stack_cap, DevStats* st, const int* sorted,
                                                                const RaySortCtl* rs, int n_smem, int* spill) {
  const int nc = rc->n_closest;
  BatchMixedSrc src{jobs, job_pass, q_closest, q_any, (rs && rs->use) ? sorted : nullptr, nc, ro, rd, hit};
  trace_loop_mixed<WIDE>(src, nc, nc + rc->n_any, &rc->work_closest, stack_cap, st, n_smem, spill);
}

// the shared-memory stack columns of a block of tb threads (n_smem entries each)
static size_t batch_smem(int n_smem, int tb) { return (size_t)tb * 2 * n_smem * sizeof(int); }

template <class K>
static int batch_grid_of(K kernel, size_t smem, int tb) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, tb, smem);
  return per_sm > 0 ? per_sm * sms : -1;
}

int batch_trace_grid(bool any_hit, int n_smem, bool wide, int tb) {
  const size_t smem = batch_smem(n_smem, tb);
  if (wide)
    return any_hit ? batch_grid_of(k_batch_trace<true, true>, smem, tb) : batch_grid_of(k_batch_trace<false, true>, smem, tb);
  return any_hit ? batch_grid_of(k_batch_trace<true, false>, smem, tb) : batch_grid_of(k_batch_trace<false, false>, smem, tb);
}

int batch_trace_mixed_grid(int n_smem, bool wide, int tb) {
  const size_t smem = batch_smem(n_smem, tb);
  return wide ? batch_grid_of(k_batch_trace_mixed<true>, smem, tb) : batch_grid_of(k_batch_trace_mixed<false>, smem, tb);
}

int launch_batch_trace_mixed(bool wide, const BatchJob* jobs, SF<int4> job_pass, const int* q_closest,
                             const int* q_any, RoundCounters* rc, SF<float4> ro, SF<float4> rd, SF<float4> hit,
                             DevStats* st, int stack_cap, int n_smem, int* spill, int grid_blocks, int tb, cudaStream_t s,
                             const int* sorted, const RaySortCtl* rs) {
  const size_t smem = batch_smem(n_smem, tb);
  if (wide)
    k_batch_trace_mixed<true><<<grid_blocks, tb, smem, s>>>(jobs, job_pass, q_closest, q_any, rc, ro, rd, hit,
                                                            stack_cap, st, sorted, rs, n_smem, spill);
  else
    k_batch_trace_mixed<false><<<grid_blocks, tb, smem, s>>>(jobs, job_pass, q_closest, q_any, rc, ro, rd, hit,
                                                             stack_cap, st, sorted, rs, n_smem, spill);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_batch_trace(bool any_hit, bool wide, const BatchJob* jobs, SF<int4> job_pass, const int* queue,
                       const int* count, int* work, SF<float4> ro, SF<float4> rd, SF<float4> hit, DevStats* st,
                       int stack_cap, int n_smem, int* spill, int grid_blocks, int tb, cudaStream_t s) {
  const size_t smem = batch_smem(n_smem, tb);
  if (any_hit && wide)
    k_batch_trace<true, true><<<grid_blocks, tb, smem, s>>>(jobs, job_pass, queue, count, work, ro, rd, hit,
                                                            stack_cap, st, n_smem, spill);
  else if (any_hit)
    k_batch_trace<true, false><<<grid_blocks, tb, smem, s>>>(jobs, job_pass, queue, count, work, ro, rd, hit,
                                                             stack_cap, st, n_smem, spill);
  else if (wide)
    k_batch_trace<false, true><<<grid_blocks, tb, smem, s>>>(jobs, job_pass, queue, count, work, ro, rd, hit,
                                                             stack_cap, st, n_smem, spill);
  else
    k_batch_trace<false, false><<<grid_blocks, tb, smem, s>>>(jobs, job_pass, queue, count, work, ro, rd, hit,
                                                              stack_cap, st, n_smem, spill);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yc
