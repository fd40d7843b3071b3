// api.cu -- the C-ABI of include/yune_cuda.h: context, scene and accumulator buffers,
// and the render-pass driver that replaces CLManager + RendererCore's OpenCL calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "yc_bdpt.h"
#include "yc_engine.h"
#include "yc_internal.h"
#include "yc_noalloc.h"
#include "yc_repack.h"
#include "yc_shade.cuh"
#include "yune_cuda.h"

namespace {

thread_local std::string g_last_error;

// device allocations (cudaMalloc) made by the context and batch buffers of this process
std::atomic<unsigned long long> g_device_allocs{0};

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

}  // namespace

namespace yc {
// the message of yc_last_error() for failures reported by the other host units (serve.cpp)
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace yc

namespace {

#define YC_CUDA(call)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail(e_ == cudaErrorMemoryAllocation ? YC_E_NOMEM : YC_E_LAUNCH,                \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                       \
  } while (0)

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    release();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    g_device_allocs.fetch_add(1, std::memory_order_relaxed);
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
  size_t bytes() const { return n * sizeof(T); }
};

struct Scene {
  DevBuf<float4> nodes, tris, shade;
  DevBuf<yc_material> mats;
  DevBuf<float2> on_ab;
  DevBuf<yc_quad_light> lights;
  yc::DevScene dev{};
  uint64_t bytes = 0;
  bool has_specular = false;   // a mirror or dielectric material: shading paths diverge most
  // yc_refit_scene: the nodes by depth (made on the first refit) and the new triangles
  DevBuf<int> refit_order;
  std::vector<int> refit_levels;
  bool refit_ready = false;
  DevBuf<yc_triangle> refit_tris;
  DevBuf<float4> refit_root;
  size_t n_node4 = 0, n_tri4 = 0, n_shade4 = 0;   // float4 records of the repacked arrays
};

struct Accum {
  DevBuf<float4> buf;
  DevBuf<float4> ldr;   // tonemapped image
  int w = 0, h = 0;
};

}  // namespace

struct yc_batch;
namespace {
void free_batch(yc_batch* b);
}

struct yc_ctx {
  int device = 0;
  std::vector<yc_batch*> batches;   // owned: destroyed with the context
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t marks[8] = {};   // yc_event_record slots
  // the any-hit trace of a round runs on side_stream beside the closest-hit trace
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::map<int, std::unique_ptr<Scene>> scenes;
  std::map<int, std::unique_ptr<Accum>> accums;
  int next_scene = 1, next_accum = 1;
  yc_cam cam{};
  bool have_cam = false;
  int tree_mode = yc::TREE_SAH_OVER_LEAVES;
  int tail_paths = -1;   // YC_OPT_TAIL: -1 = one resident launch of the tail kernel, 0 = off
  int mixed_trace = 1;   // YC_OPT_MIXED_TRACE: one traversal launch per round for both ray kinds
  std::vector<yc_bvh_node> built_nodes;   // the last yc_bvh_build
  int built_depth = 0;
  int rs_ob = 3, rs_db = 2;       // YC_OPT_RAY_SORT: origin / direction bits per axis of the sort key
  int rs_threshold = 65536;       // YC_OPT_RAY_SORT_MIN: rounds with fewer rays are not sorted
  int ss_threshold = 65536;       // YC_OPT_SHADE_SORT_MIN: per-pass shade queues this long are sorted
  DevBuf<int> ss_keys, ss_sorted;
  DevBuf<yc::SortCtl> ss_ctl;
  size_t ss_cap = 0;
  // ray sort of the per-pass path (raysort.cu)
  DevBuf<unsigned> rs_keys, rs_hist, rs_cursor, rs_blk;
  DevBuf<int> rs_sorted;
  DevBuf<yc::RaySortCtl> rs_ctl;
  size_t rs_cap = 0;
  // wavefront buffers, sized for the largest image seen
  size_t cap_paths = 0;
  DevBuf<float4> rec;                // path records, PS_STRIDE float4 per slot
  DevBuf<int> q[4];                  // closest/any for two rounds
  DevBuf<yc::RoundCounters> rc;      // two round-counter blocks
  DevBuf<yc::DevStats> stats;
  yc::RoundCounters* rc_host = nullptr;   // pinned
  unsigned long long* overflow_host = nullptr;   // pinned: DevStats::call_overflow read back
  int max_rounds = 1000000;   // YC_OPT_MAX_ROUNDS: rounds one pass may take
  int stack_limit = 0;        // YC_OPT_STACK_LIMIT: traversal stack entries allowed (0 = any)
  int stack_smem = 12;        // YC_OPT_STACK_SMEM: per-pass walk-stack entries in shared memory
  int repack_device = 1;      // YC_OPT_REPACK: the upload's repack of tree mode 1 on the device
  DevBuf<int> pass_spill;     // the deeper entries of the per-pass walks (with stack_smem)
  int logic_grid = 0;
  int sm_count = 0;
  float last_ms = 0.0f;
  // per-kernel event timing
  bool profile = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, size_t>> ev_marks;   // kind, index of the start event
  yc_kernel_times ktimes{};
  DevBuf<char> flush_buf;
  // BDPT subpath vertices
  DevBuf<float4> bd_lv, bd_ev;
  size_t bd_cap = 0, bd_ev_cap = 0;   // light / eye vertex records (the MIS tracer has no eye records)
  // direct queries
  DevBuf<float> q_rays;
  DevBuf<int> q_tri;
  DevBuf<float> q_t;
  DevBuf<int> q_work;
};

namespace {

int ensure_paths(yc_ctx* c, size_t n) {
  if (n <= c->cap_paths) return 0;
  YC_CUDA(c->rec.alloc(n * yc::PS_STRIDE));
  for (auto& b : c->q) YC_CUDA(b.alloc(n));
  c->cap_paths = n;
  return 0;
}

// scenes with fewer triangles are traced in queue order by yc_render_pass
constexpr int kRaySortMinTris = 4096;
// frames with fewer pixels are shaded in queue order by yc_render_pass
constexpr size_t kShadeSortMinPixels = 1u << 19;

// FNV-1a over the 64-bit words of the repacked node, stream and shading arrays, the root
// box and the root link and test (yc_scene_layout, yc_scene_digest)
uint64_t layout_digest(const float4* nodes, size_t n_nodes, const float4* tris, size_t n_tris, const float4* shade,
                       size_t n_shade, float4 root_lo, float4 root_hi, int root_link, int root_test) {
  uint64_t h = 0xcbf29ce484222325ull;
  // the 64-bit words are copied out of the float4 bytes (memcpy), not read through a
  // uint64_t pointer: an aliased read of a float4 object is undefined, and an optimising
  // compiler may then drop the stores that fill the array (the root box below)
  auto words = [&h](const float4* p, size_t n) {
    const unsigned char* bytes = reinterpret_cast<const unsigned char*>(p);
    h = (h ^ (uint64_t)n) * 0x100000001b3ull;
    for (size_t i = 0; i < 2 * n; ++i) {
      uint64_t w;
      std::memcpy(&w, bytes + 8 * i, 8);
      h = (h ^ w) * 0x100000001b3ull;
    }
  };
  words(nodes, n_nodes);
  words(tris, n_tris);
  words(shade, n_shade);
  const float4 root[2] = {root_lo, root_hi};
  words(root, 2);
  h = (h ^ (uint64_t)(uint32_t)root_link) * 0x100000001b3ull;
  h = (h ^ (uint64_t)(uint32_t)root_test) * 0x100000001b3ull;
  return h;
}

// the per-pass walks' stack spill area: n ints
int ensure_pass_spill(yc_ctx* c, size_t n) {
  if (n > c->pass_spill.n) YC_CUDA(c->pass_spill.alloc(n));
  return 0;
}

// key, histogram and sorted-list buffers of the per-pass ray sort, for n rays
int ensure_raysort(yc_ctx* c, size_t n) {
  if (!c->rs_hist.p) {
    const size_t bins = (size_t)yc::raysort_bins(3, 2);   // the largest key allowed (16 bits)
    YC_CUDA(c->rs_hist.alloc(bins));
    YC_CUDA(c->rs_cursor.alloc(bins));
    YC_CUDA(c->rs_blk.alloc(64));
    YC_CUDA(c->rs_ctl.alloc(1));
    YC_CUDA(cudaMemsetAsync(c->rs_hist.p, 0, c->rs_hist.bytes(), c->stream));
    YC_CUDA(cudaMemsetAsync(c->rs_ctl.p, 0, sizeof(yc::RaySortCtl), c->stream));
  }
  if (n > c->rs_cap) {
    YC_CUDA(c->rs_keys.alloc(n));
    YC_CUDA(c->rs_sorted.alloc(n));
    c->rs_cap = n;
  }
  return 0;
}

// key and sorted-list buffers of the per-pass shade-queue sort, for n paths
int ensure_shadesort(yc_ctx* c, size_t n) {
  if (!c->ss_ctl.p) YC_CUDA(c->ss_ctl.alloc(1));
  if (n > c->ss_cap) {
    YC_CUDA(c->ss_keys.alloc(n));
    YC_CUDA(c->ss_sorted.alloc(n));
    c->ss_cap = n;
  }
  return 0;
}

// event pairs around kernel launches (profiling only)
enum { K_RAYGEN = 0, K_EXTEND = 1, K_OCCL = 2, K_LOGIC = 3, K_SORT = 4, K_TAIL = 5, K_TRACE = 6, K_RAYSORT = 7 };
cudaEvent_t next_event(yc_ctx* c) {
  if (c->ev_used == c->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    c->ev_pool.push_back(e);
  }
  return c->ev_pool[c->ev_used++];
}
struct KTimer {
  yc_ctx* c;
  int kind;
  size_t idx = 0;
  bool on;
  KTimer(yc_ctx* c_, int k, bool allowed = true) : c(c_), kind(k), on(c_->profile && allowed) {
    if (!on) return;
    idx = c->ev_used;
    cudaEvent_t e = next_event(c);
    if (!e) { on = false; return; }
    cudaEventRecord(e, c->stream);
  }
  ~KTimer() {
    if (!on) return;
    cudaEvent_t e = next_event(c);
    if (!e) return;
    cudaEventRecord(e, c->stream);
    c->ev_marks.emplace_back(kind, idx);
  }
};
void collect_events(yc_ctx* c) {
  if (c->ev_marks.empty()) { c->ev_used = 0; return; }
  cudaStreamSynchronize(c->stream);
  for (auto& m : c->ev_marks) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, c->ev_pool[m.second], c->ev_pool[m.second + 1]);
    switch (m.first) {
      case K_RAYGEN: c->ktimes.raygen_ms += ms; c->ktimes.raygen_launches++; break;
      case K_EXTEND: c->ktimes.extend_ms += ms; c->ktimes.extend_launches++; break;
      case K_OCCL: c->ktimes.occlusion_ms += ms; c->ktimes.occlusion_launches++; break;
      case K_SORT: c->ktimes.sort_ms += ms; c->ktimes.sort_launches++; break;
      case K_TAIL: c->ktimes.tail_ms += ms; c->ktimes.tail_launches++; break;
      case K_TRACE: c->ktimes.trace_ms += ms; c->ktimes.trace_launches++; break;
      case K_RAYSORT: c->ktimes.raysort_ms += ms; c->ktimes.raysort_launches++; break;
      default: c->ktimes.logic_ms += ms; c->ktimes.logic_launches++; break;
    }
  }
  c->ev_marks.clear();
  c->ev_used = 0;
}

yc::PathState path_state(yc_ctx* c) { return yc::path_state_at(c->rec.p); }

Scene* find_scene(yc_ctx* c, int id) {
  auto it = c->scenes.find(id);
  return it == c->scenes.end() ? nullptr : it->second.get();
}
Accum* find_accum(yc_ctx* c, int id) {
  auto it = c->accums.find(id);
  return it == c->accums.end() ? nullptr : it->second.get();
}

int validate_cfg(const yc_pass_cfg* cfg) {
  if (!cfg) return fail(YC_E_INVALID, "cfg is NULL");
  if (cfg->integrator != YC_UDPT && cfg->integrator != YC_BDPT && cfg->integrator != YC_BDPT_MIS)
    return fail(YC_E_INVALID, "unknown integrator");
  if (cfg->max_depth < 0) return fail(YC_E_INVALID, "max_depth < 0");
  if (cfg->block_x < 1 || cfg->block_y < 1 || cfg->block < 0 || cfg->block >= cfg->block_x * cfg->block_y)
    return fail(YC_E_INVALID, "bad block tiling");
  return 0;
}

// The kernel arguments of one pass (`pathtracer`, udpt.cl:158-160): scene, camera,
// accumulator, the tile of cfg->block (udpt.cl:166-167, src/RendererCore.cpp:146-150) and
// the options the reference bakes into its kernel text. yc_render_pass and
// yc_render_pass_noalloc both build their passes here. The scene's traversal depth is
// capped by YC_OPT_STACK_LIMIT (a deeper walk then overflows and the call fails).
yc::PassParams pass_params(const yc_ctx* c, const Scene* sc, const Accum* ac, uint32_t rand_seed, int reset,
                           int gi_check, const yc_pass_cfg* cfg) {
  yc::PassParams pp{};
  pp.sc = sc->dev;
  if (c->stack_limit > 0) pp.sc.depth = std::min(pp.sc.depth, c->stack_limit - 2);
  pp.cam = c->cam;
  pp.accum = ac->buf.p;
  pp.width = ac->w;
  pp.height = ac->h;
  pp.aspect = yc::frame_aspect(ac->w, ac->h);
  pp.tile_w = (int)std::ceil((float)ac->w / cfg->block_x);
  pp.tile_h = (int)std::ceil((float)ac->h / cfg->block_y);
  pp.off_x = (int)(std::ceil((float)ac->w / cfg->block_x) * (float)(cfg->block % cfg->block_x));
  pp.off_y = (int)(std::ceil((float)ac->h / cfg->block_y) * (float)(cfg->block / cfg->block_x));
  pp.rand_seed = rand_seed;
  pp.reset = reset;
  pp.gi_check = gi_check;
  pp.mis = cfg->mis;
  pp.rr_threshold = cfg->rr_threshold;
  pp.max_depth = cfg->max_depth;
  pp.brdf_model = cfg->brdf_model;
  pp.mis_lobe_fix = cfg->mis_lobe_fix;
  return pp;
}

// Per-call error state: the call's stack-overflow count is cleared when a render call
// starts and read back when it ends (the reference surfaces every failure of a pass as an
// error, src/CLManager.cpp:755-855; a walk that overflowed its stack gave a wrong hit).
int begin_call_checks(yc_ctx* c) {
  YC_CUDA(cudaMemsetAsync(&c->stats.p->call_overflow, 0, sizeof(unsigned long long), c->stream));
  return 0;
}
int queue_call_checks(yc_ctx* c) {
  YC_CUDA(cudaMemcpyAsync(c->overflow_host, &c->stats.p->call_overflow, sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, c->stream));
  return 0;
}
// after the stream has been synchronised
int end_call_checks(yc_ctx* c) {
  if (*c->overflow_host)
    return fail(YC_E_OVERFLOW, std::to_string(*c->overflow_host) +
                                   " traversals reached the stack bound (their hits are wrong); the scene's hierarchy "
                                   "is deeper than YC_OPT_STACK_LIMIT or the batch's stack_cap allows");
  return 0;
}

// Runs one pass (all rounds) on the context stream; the host polls the queue sizes
// every few rounds. YC_E_TIMEOUT when paths are still live after YC_OPT_MAX_ROUNDS rounds.
int run_pass(yc_ctx* c, Scene* sc, Accum* ac, uint32_t rand_seed, int reset, int gi_check, const yc_pass_cfg* cfg) {
  const bool bdpt = cfg->integrator != YC_UDPT;
  const bool bdpt_mis = cfg->integrator == YC_BDPT_MIS;
  if (bdpt && (cfg->bdpt_bounces < 2 || cfg->bdpt_bounces > 32)) return fail(YC_E_INVALID, "bdpt_bounces must be 2..32");
  if (bdpt_mis && cfg->bdpt_bounces < 3) return fail(YC_E_INVALID, "bdpt_bounces must be 3..32 with YC_BDPT_MIS");
  const int W = ac->w, H = ac->h;
  int rc_ = ensure_paths(c, (size_t)W * H);
  if (rc_) return rc_;
  const yc::PassParams pp = pass_params(c, sc, ac, rand_seed, reset, gi_check, cfg);
  const yc::DevScene& dsc = pp.sc;   // the scene as the kernels walk it (stack limit applied)
  const yc::PathState ps = path_state(c);
  yc::BdptBuffers bb{};
  if (bdpt) {
    const size_t need = (size_t)W * H * 4 * cfg->bdpt_bounces;
    if (c->bd_cap < need) {
      YC_CUDA(c->bd_lv.alloc(need));
      c->bd_cap = need;
    }
    if (!bdpt_mis && c->bd_ev_cap < need) {
      YC_CUDA(c->bd_ev.alloc(need));
      c->bd_ev_cap = need;
    }
    bb.lv = c->bd_lv.p;
    bb.ev = c->bd_ev.p;
    bb.N = (size_t)W * H;
    bb.bounces = cfg->bdpt_bounces;
  }
  yc::RoundCounters* rc = c->rc.p;
  YC_CUDA(cudaMemsetAsync(rc, 0, 2 * sizeof(yc::RoundCounters), c->stream));
  {
    KTimer kt(c, K_RAYGEN);
    if (bdpt_mis) yc::launch_raygen_bdpt_mis(pp, ps, bb, c->q[0].p, rc + 0, c->stats.p, c->stream);
    else if (bdpt) yc::launch_raygen_bdpt(pp, ps, bb, c->q[0].p, rc + 0, c->stats.p, c->stream);
    else yc::launch_raygen(pp, ps, c->q[0].p, rc + 0, c->stats.p, c->stream);
  }
  YC_CUDA(cudaPeekAtLastError());
  const bool mixed = c->mixed_trace != 0;
  // (a walk through a scene of a few thousand triangles is a handful of boxes: sorting
  // its rays costs more than it saves)
  const bool raysort = mixed && (c->rs_ob + c->rs_db) > 0 && c->rs_threshold > 0 &&
                       (size_t)W * H >= (size_t)c->rs_threshold && dsc.n_tri >= kRaySortMinTris;
  yc::RaySortBufs rsb{};
  if (raysort) {
    if (int e = ensure_raysort(c, (size_t)W * H)) return e;
    rsb = yc::RaySortBufs{c->rs_keys.p, nullptr, c->rs_hist.p, c->rs_cursor.p, c->rs_blk.p, c->rs_sorted.p, c->rs_ctl.p,
                          c->rs_ob, c->rs_db, 0, c->rs_threshold};
  }
  // shade-queue sort by phase and material class before the logic kernel (unidirectional
  // passes whose frame can fill a sorted queue, in scenes with a mirror or dielectric:
  // with diffuse and glossy materials alone the paths' shading code differs too little
  // for the sort to pay, measured)
  // BDPT paths are sorted by their state in any scene (light subpath, eye subpath, NEE and
  // connection steps run different code). The sort's three launches per round pay back
  // from frames of about half a million paths (measured: 1024x1024 and 3840x2160 gain,
  // 512x512 loses).
  // The MIS tracer's states differ more (light subpath, next event, connections with four
  // densities each, continuation): its sort pays from the option's threshold on (measured:
  // 1024x1024 at 662 against 448 Mrays/s unsorted).
  const bool shadesort = (bdpt || sc->has_specular) && c->ss_threshold > 0 &&
                         (size_t)W * H >= (bdpt_mis ? (size_t)c->ss_threshold
                                                    : std::max((size_t)c->ss_threshold, kShadeSortMinPixels));
  if (shadesort)
    if (int e = ensure_shadesort(c, (size_t)W * H)) return e;
  const int grid_c = yc::trace_grid_blocks(false, dsc.depth, dsc.wide != 0);
  const int grid_a = yc::trace_grid_blocks(true, dsc.depth, dsc.wide != 0);
  // the mixed trace's walk stacks: c->stack_smem entries in shared memory, the rest spilled
  const int cap = yc::trace_stack_cap(dsc.depth);
  const int n_smem = (mixed && c->stack_smem < cap) ? c->stack_smem : 0;   // 0: the whole stack
  const int grid_m = mixed ? yc::trace_mixed_grid_blocks(dsc.depth, dsc.wide != 0, n_smem) : 1;
  if (n_smem > 0 && grid_m > 0)
    if (int e = ensure_pass_spill(c, (size_t)grid_m * yc::TRACE_TB_PASS * 2 * (size_t)(cap - n_smem))) return e;
  if (grid_c <= 0 || grid_a <= 0 || grid_m <= 0)
    return fail(YC_E_LAUNCH, "trace kernel cannot be resident (stack too deep)");
  int tail_grid = 0, tail_at = 0;
  if (!bdpt && c->tail_paths != 0) {
    const int capacity = yc::tail_capacity(dsc, &tail_grid);
    tail_at = c->tail_paths < 0 ? capacity : std::min(c->tail_paths, capacity);
  }
  int cur = 0;
  const int check_every = 6;
  bool finished = false;
  for (int round = 0; round < c->max_rounds; ++round) {
    int* in_c = c->q[2 * cur].p;
    int* in_a = c->q[2 * cur + 1].p;
    int* out_c = c->q[2 * (1 - cur)].p;
    int* out_a = c->q[2 * (1 - cur) + 1].p;
    yc::RoundCounters* rin = rc + cur;
    yc::RoundCounters* rout = rc + (1 - cur);
    int e1, e2;
    if (mixed) {   // both ray kinds of the round in one launch
      if (raysort) {
        KTimer kt(c, K_RAYSORT);
        if (yc::launch_raysort(dsc, in_c, in_a, rin, ps.ro, ps.rd, rsb, c->logic_grid, c->stream))
          return fail(YC_E_LAUNCH, std::string("ray sort: ") + cudaGetErrorString(cudaGetLastError()));
      }
      KTimer kt(c, K_TRACE);
      if (yc::launch_trace_mixed(dsc, in_c, in_a, rin, ps.ro, ps.rd, ps.hit, c->stats.p, grid_m, c->stream,
                                 raysort ? rsb.sorted : nullptr, raysort ? rsb.ctl : nullptr, n_smem,
                                 n_smem > 0 ? c->pass_spill.p : nullptr))
        return fail(YC_E_LAUNCH, std::string("trace kernel: ") + cudaGetErrorString(cudaGetLastError()));
    }
    // otherwise the two traces of a round are independent: the any-hit one runs on the
    // side stream so that each fills the SMs the other's last rays leave idle (sequential
    // when profiling, so each kernel's events time it alone)
    const bool overlap = !c->profile && !mixed;
    cudaStream_t s_any = overlap ? c->side_stream : c->stream;
    if (overlap) {
      YC_CUDA(cudaEventRecord(c->ev_fork, c->stream));
      YC_CUDA(cudaStreamWaitEvent(c->side_stream, c->ev_fork, 0));
    }
    if (!mixed) {
      {
        KTimer kt(c, K_EXTEND);
        e1 = yc::launch_trace(dsc, false, in_c, &rin->n_closest, &rin->work_closest, ps.ro, ps.rd, ps.hit,
                              c->stats.p, grid_c, c->stream);
      }
      if (e1) return fail(YC_E_LAUNCH, std::string("extend kernel: ") + cudaGetErrorString(cudaGetLastError()));
      {
        KTimer kt(c, K_OCCL);
        e2 = yc::launch_trace(dsc, true, in_a, &rin->n_any, &rin->work_any, ps.ro, ps.rd, ps.hit, c->stats.p,
                              grid_a, s_any);
      }
      if (e2) return fail(YC_E_LAUNCH, std::string("occlusion kernel: ") + cudaGetErrorString(cudaGetLastError()));
    }
    if (overlap) {
      YC_CUDA(cudaEventRecord(c->ev_join, c->side_stream));
      YC_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    }
    YC_CUDA(cudaMemsetAsync(rout, 0, sizeof(yc::RoundCounters), c->stream));
    if (shadesort) {
      KTimer kt(c, K_SORT);
      YC_CUDA(cudaMemsetAsync(c->ss_ctl.p, 0, sizeof(yc::SortCtl), c->stream));
      yc::launch_pass_sort(dsc, bdpt, ps, in_c, in_a, rin, c->ss_keys.p, c->ss_sorted.p, c->ss_ctl.p,
                           c->ss_threshold, c->logic_grid, c->stream);
    }
    {
      KTimer kt(c, K_LOGIC);
      const int* sorted = shadesort ? c->ss_sorted.p : nullptr;
      const yc::SortCtl* sctl = shadesort ? c->ss_ctl.p : nullptr;
      if (bdpt_mis)
        yc::launch_logic_bdpt_mis(pp, ps, bb, in_c, in_a, rin, out_c, out_a, rout, c->stats.p, c->logic_grid,
                                  c->stream, sorted, sctl);
      else if (bdpt)
        yc::launch_logic_bdpt(pp, ps, bb, in_c, in_a, rin, out_c, out_a, rout, c->stats.p, c->logic_grid, c->stream,
                              sorted, sctl);
      else yc::launch_logic(pp, ps, in_c, in_a, rin, out_c, out_a, rout, c->stats.p, c->logic_grid, c->stream,
                            sorted, sctl);
    }
    if (tail_at > 0) {
      KTimer kt(c, K_TAIL);
      if (yc::launch_tail(pp, ps, out_c, out_a, rout, tail_at, c->stats.p, tail_grid, c->stream))
        return fail(YC_E_LAUNCH, std::string("tail kernel: ") + cudaGetErrorString(cudaGetLastError()));
    }
    YC_CUDA(cudaPeekAtLastError());
    c->ktimes.rounds++;
    cur = 1 - cur;
    if ((round + 1) % check_every == 0 || round + 1 == c->max_rounds) {
      YC_CUDA(cudaMemcpyAsync(c->rc_host, rc + cur, sizeof(yc::RoundCounters), cudaMemcpyDeviceToHost, c->stream));
      YC_CUDA(cudaStreamSynchronize(c->stream));
      if (c->rc_host->n_closest == 0 && c->rc_host->n_any == 0) { finished = true; break; }
    }
  }
  if (!finished)
    return fail(YC_E_TIMEOUT, "pass not finished after " + std::to_string(c->max_rounds) + " rounds (" +
                                  std::to_string(c->rc_host->n_closest + c->rc_host->n_any) +
                                  " rays still queued; YC_OPT_MAX_ROUNDS)");
  return 0;
}

}  // namespace

extern "C" {

const char* yc_last_error(void) { return g_last_error.c_str(); }

int yc_create(int device, yc_ctx** out) {
  if (!out) return fail(YC_E_INVALID, "out is NULL");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return fail(YC_E_NODEVICE, "no CUDA device");
  if (device < 0 || device >= n) return fail(YC_E_INVALID, "device index out of range");
  YC_CUDA(cudaSetDevice(device));
  yc_ctx* c = new (std::nothrow) yc_ctx;
  if (!c) return fail(YC_E_NOMEM, "host allocation failed");
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = c->rc.alloc(2);
  if (e == cudaSuccess) e = c->stats.alloc(1);
  if (e == cudaSuccess) e = cudaMallocHost(&c->rc_host, sizeof(yc::RoundCounters));
  if (e == cudaSuccess) e = cudaMallocHost(&c->overflow_host, sizeof(unsigned long long));
  if (e == cudaSuccess) e = c->q_work.alloc(1);
  if (e == cudaSuccess) e = cudaMemset(c->stats.p, 0, sizeof(yc::DevStats));
  if (e != cudaSuccess) {
    yc_destroy(c);
    return fail(YC_E_LAUNCH, std::string("context setup: ") + cudaGetErrorString(e));
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  c->logic_grid = std::max(1, c->sm_count) * 4;
  *out = c;
  return YC_OK;
}

int yc_destroy(yc_ctx* c) {
  if (!c) return YC_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (yc_batch* b : c->batches) free_batch(b);   // batches never outlive their context
  c->batches.clear();
  c->scenes.clear();
  c->accums.clear();
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  c->ev_pool.clear();
  if (c->rc_host) cudaFreeHost(c->rc_host);
  if (c->overflow_host) cudaFreeHost(c->overflow_host);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t& e : c->marks)
    if (e) cudaEventDestroy(e);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->side_stream) {
    cudaStreamSynchronize(c->side_stream);
    cudaStreamDestroy(c->side_stream);
  }
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return YC_OK;
}

int yc_synchronize(yc_ctx* c) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YC_OK;
}

int yc_upload_scene(yc_ctx* c, const yc_triangle* tris, int n_tri, const yc_material* mats, int n_mat,
                    const yc_bvh_node* nodes, int n_node, const yc_quad_light* lights, int n_light, int* scene_id) {
  if (!c || !scene_id) return fail(YC_E_INVALID, "ctx or scene_id is NULL");
  if (n_tri < 0 || n_mat < 0 || n_node < 0) return fail(YC_E_INVALID, "negative count");
  if ((n_tri > 0 && !tris) || (n_mat > 0 && !mats) || (n_node > 0 && !nodes))
    return fail(YC_E_INVALID, "NULL array with non-zero count");
  if (n_light < 1 || n_light > yc::MAX_LIGHTS || !lights) return fail(YC_E_INVALID, "need 1..16 lights");
  {
    std::string err;
    if (yc::check_materials(tris, n_tri, n_mat, err)) return fail(YC_E_INVALID, err);
  }
  yc::Repacked rp;
  yc::DevRepackPlan plan;
  std::string err;
  // the repack: on the device for tree mode 1 (YC_OPT_REPACK), where a scene has two
  // reachable leaves or more; otherwise (and for the trivial scenes) on the host
  int on_device = 0;
  if (c->repack_device && c->tree_mode == yc::TREE_SAH_OVER_LEAVES) {
    on_device = yc::plan_device_repack(nodes, n_node, n_tri, plan, err);
    if (on_device < 0) return fail(YC_E_INVALID, err);
  }
  if (!on_device && yc::repack_scene(tris, n_tri, nodes, n_node, c->tree_mode, rp, err)) return fail(YC_E_INVALID, err);
  const size_t n_node4 = on_device ? 4 * (plan.leaf_node.size() - 1) : rp.nodes.size();
  const size_t n_tri4 = on_device ? 3 * plan.slots : rp.tris.size();
  const size_t n_shade4 = on_device ? 4 * (size_t)n_tri : rp.shade.size();
  std::unique_ptr<Scene> s(new (std::nothrow) Scene);
  if (s)
    for (int i = 0; i < n_mat; ++i) s->has_specular = s->has_specular || mats[i].is_specular != 0;
  if (!s) return fail(YC_E_NOMEM, "host allocation failed");
  YC_CUDA(cudaSetDevice(c->device));
  YC_CUDA(s->nodes.alloc(std::max<size_t>(n_node4, 4)));
  YC_CUDA(s->tris.alloc(std::max<size_t>(n_tri4, 3)));
  YC_CUDA(s->shade.alloc(std::max<size_t>(n_shade4, 4)));
  YC_CUDA(s->mats.alloc(std::max(n_mat, 1)));
  YC_CUDA(s->on_ab.alloc(std::max(n_mat, 1)));
  YC_CUDA(s->lights.alloc(yc::MAX_LIGHTS));
  s->n_node4 = n_node4;
  s->n_tri4 = n_tri4;
  s->n_shade4 = n_shade4;
  if (on_device) {
    int depth = 0;
    const int r = yc::repack_device(tris, n_tri, nodes, n_node, plan, s->nodes.p, s->tris.p, s->shade.p, depth,
                                    c->stream, err);
    if (r) return fail(r == -2 ? YC_E_NOMEM : YC_E_LAUNCH, err);
    rp.root_link = 0;   // the root is the first node (two leaves or more)
    rp.root_test = 1;
    rp.depth = depth;
    rp.wide = 0;
    rp.root_lo = plan.root_lo;
    rp.root_hi = plan.root_hi;
  }
  if (!rp.nodes.empty())
    YC_CUDA(cudaMemcpyAsync(s->nodes.p, rp.nodes.data(), rp.nodes.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
  if (!rp.tris.empty())
    YC_CUDA(cudaMemcpyAsync(s->tris.p, rp.tris.data(), rp.tris.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
  if (!rp.shade.empty())
    YC_CUDA(cudaMemcpyAsync(s->shade.p, rp.shade.data(), rp.shade.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
  std::vector<float2> on_ab(std::max(n_mat, 1), float2{0.0f, 0.0f});
  for (int i = 0; i < n_mat; ++i) on_ab[i] = yc::oren_nayar_ab(mats[i].alpha_x);
  if (n_mat > 0)
    YC_CUDA(cudaMemcpyAsync(s->mats.p, mats, n_mat * sizeof(yc_material), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaMemcpyAsync(s->on_ab.p, on_ab.data(), on_ab.size() * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaMemcpyAsync(s->lights.p, lights, n_light * sizeof(yc_quad_light), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  yc::DevScene& d = s->dev;
  d.nodes = s->nodes.p;
  d.tris = s->tris.p;
  d.shade = s->shade.p;
  d.mats = s->mats.p;
  d.lights = s->lights.p;
  d.on_ab = s->on_ab.p;
  d.n_lights = n_light;
  d.n_tri = n_tri;
  d.n_mat = n_mat;
  d.root_link = rp.root_link;
  d.root_test = rp.root_test;
  d.depth = rp.depth;
  d.wide = rp.wide;
  d.root_lo = rp.root_lo;
  d.root_hi = rp.root_hi;
  s->bytes = s->nodes.bytes() + s->tris.bytes() + s->shade.bytes() + s->mats.bytes() + s->on_ab.bytes() +
             s->lights.bytes();
  const int id = c->next_scene++;
  c->scenes[id] = std::move(s);
  *scene_id = id;
  return YC_OK;
}

int yc_scene_layout(const yc_triangle* tris, int n_tri, int n_mat, const yc_bvh_node* nodes, int n_node,
                    int tree_mode, yc_scene_layout_info* out) {
  if (!out) return fail(YC_E_INVALID, "out is NULL");
  if (n_tri < 0 || n_mat < 0 || n_node < 0) return fail(YC_E_INVALID, "negative count");
  if ((n_tri > 0 && !tris) || (n_node > 0 && !nodes)) return fail(YC_E_INVALID, "NULL array with non-zero count");
  if (tree_mode != yc::TREE_REFERENCE && tree_mode != yc::TREE_SAH_OVER_LEAVES && tree_mode != yc::TREE_WIDE4)
    return fail(YC_E_INVALID, "bad tree mode");
  {
    std::string err;
    if (yc::check_materials(tris, n_tri, n_mat, err)) return fail(YC_E_INVALID, err);
  }
  yc::Repacked rp;
  std::string err;
  if (yc::repack_scene(tris, n_tri, nodes, n_node, tree_mode, rp, err)) return fail(YC_E_INVALID, err);
  // the allocations of yc_upload_scene
  out->node_bytes = std::max<size_t>(rp.nodes.size(), 4) * sizeof(float4);
  out->stream_bytes = std::max<size_t>(rp.tris.size(), 3) * sizeof(float4);
  out->shade_bytes = std::max<size_t>(rp.shade.size(), 4) * sizeof(float4);
  out->device_bytes = out->node_bytes + out->stream_bytes + out->shade_bytes +
                      (uint64_t)std::max(n_mat, 1) * (sizeof(yc_material) + sizeof(float2)) +
                      yc::MAX_LIGHTS * sizeof(yc_quad_light);
  out->digest = layout_digest(rp.nodes.data(), rp.nodes.size(), rp.tris.data(), rp.tris.size(), rp.shade.data(),
                              rp.shade.size(), rp.root_lo, rp.root_hi, rp.root_link, rp.root_test);
  out->depth = rp.depth;
  out->wide = rp.wide;
  return YC_OK;
}

int yc_walk_counts(const yc_triangle* tris, int n_tri, const yc_bvh_node* nodes, int n_node, int tree_mode,
                   const float* rays9, int n, int any_hit, uint64_t* boxes, uint64_t* tris_tested, int* tri_out,
                   float* t_out) {
  if (!boxes || !tris_tested || n < 0 || (n > 0 && !rays9)) return fail(YC_E_INVALID, "bad argument");
  if (tree_mode != yc::TREE_REFERENCE && tree_mode != yc::TREE_SAH_OVER_LEAVES && tree_mode != yc::TREE_WIDE4)
    return fail(YC_E_INVALID, "bad tree mode");
  yc::Repacked rp;
  std::string err;
  if (yc::repack_scene(tris, n_tri, nodes, n_node, tree_mode, rp, err)) return fail(YC_E_INVALID, err);
  if (yc::walk_counts_host(rp, rays9, n, any_hit != 0, boxes, tris_tested, tri_out, t_out, err))
    return fail(YC_E_INVALID, err);
  return YC_OK;
}

int yc_bvh_build(yc_ctx* c, const yc_triangle* tris, int n_tri, int bins, int leaf_max, int* n_node, int* depth) {
  if (!c || n_tri < 0 || (n_tri > 0 && !tris) || leaf_max < 1 || leaf_max > 10 || bins < 0 || bins > 256)
    return fail(YC_E_INVALID, "yc_bvh_build: bad argument");
  YC_CUDA(cudaSetDevice(c->device));
  DevBuf<yc_triangle> dt;
  YC_CUDA(dt.alloc(std::max(n_tri, 1)));
  if (n_tri) YC_CUDA(cudaMemcpyAsync(dt.p, tris, n_tri * sizeof(yc_triangle), cudaMemcpyHostToDevice, c->stream));
  int d = 0;
  bool too_deep = false;
  try {
    YC_CUDA(yc::bvh_build_device(dt.p, n_tri, bins, leaf_max, c->stream, c->built_nodes, d, too_deep));
  } catch (const std::bad_alloc&) {
    return fail(YC_E_NOMEM, "yc_bvh_build: host allocation failed");
  }
  if (too_deep) {
    c->built_nodes.clear();
    return fail(YC_E_INVALID, "yc_bvh_build: more than leaf_max triangles share one centroid (the tree would not end)");
  }
  c->built_depth = d;
  if (n_node) *n_node = (int)c->built_nodes.size();
  if (depth) *depth = d;
  return YC_OK;
}

int yc_bvh_copy_nodes(yc_ctx* c, yc_bvh_node* out, int capacity) {
  if (!c || !out) return fail(YC_E_INVALID, "NULL argument");
  if (capacity < (int)c->built_nodes.size()) return fail(YC_E_INVALID, "yc_bvh_copy_nodes: capacity below the node count");
  std::memcpy(out, c->built_nodes.data(), c->built_nodes.size() * sizeof(yc_bvh_node));
  return YC_OK;
}

int yc_set_lights(yc_ctx* c, int scene_id, const yc_quad_light* lights, int n_light) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  Scene* s = find_scene(c, scene_id);
  if (!s) return fail(YC_E_NOTFOUND, "unknown scene");
  if (n_light < 1 || n_light > yc::MAX_LIGHTS || !lights) return fail(YC_E_INVALID, "need 1..16 lights");
  YC_CUDA(cudaMemcpyAsync(s->lights.p, lights, n_light * sizeof(yc_quad_light), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  s->dev.n_lights = n_light;
  return YC_OK;
}

}  // extern "C"

namespace {

// the nodes of scene s grouped by depth, deepest first (from the links of its node array)
int make_refit_plan(yc_ctx* c, Scene* s) {
  const bool wide = s->dev.wide != 0;
  const size_t per = wide ? 8 : 4;
  const size_t n = s->dev.root_link >= 0 && s->dev.root_link != yc::LINK_NONE ? s->nodes.n / per : 0;
  std::vector<int> links(n * (wide ? 4 : 2));
  if (n > 0)   // the link words of each node record, gathered with one strided copy
    YC_CUDA(cudaMemcpy2DAsync(links.data(), (wide ? 4 : 2) * sizeof(int), s->nodes.p + (per - (wide ? 2 : 1)),
                              per * sizeof(float4), (wide ? 4 : 2) * sizeof(int), n, cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  const int nc = wide ? 4 : 2;
  std::vector<int> depth(n, -1);
  std::vector<int> q;
  if (n > 0) {
    depth[s->dev.root_link] = 0;
    q.push_back(s->dev.root_link);
  }
  int max_d = 0;
  for (size_t i = 0; i < q.size(); ++i) {
    const int node = q[i];
    for (int k = 0; k < nc; ++k) {
      const int l = links[(size_t)node * nc + k];
      if (l >= 0 && l != yc::LINK_NONE && (size_t)l < n && depth[l] < 0) {
        depth[l] = depth[node] + 1;
        max_d = std::max(max_d, depth[l]);
        q.push_back(l);
      }
    }
  }
  std::vector<int> order;
  order.reserve(q.size());
  s->refit_levels.clear();
  for (int d = max_d; d >= 0 && !q.empty(); --d) {
    s->refit_levels.push_back((int)order.size());
    for (int node : q)
      if (depth[node] == d) order.push_back(node);
  }
  s->refit_levels.push_back((int)order.size());
  YC_CUDA(s->refit_order.alloc(std::max<size_t>(order.size(), 1)));
  if (!order.empty())
    YC_CUDA(cudaMemcpyAsync(s->refit_order.p, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice,
                            c->stream));
  YC_CUDA(s->refit_root.alloc(2));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  s->refit_ready = true;
  return 0;
}

}  // namespace

extern "C" {

int yc_refit_scene(yc_ctx* c, int scene_id, const yc_triangle* tris, int n_tri) {
  if (!c || (n_tri > 0 && !tris)) return fail(YC_E_INVALID, "NULL argument");
  Scene* s = find_scene(c, scene_id);
  if (!s) return fail(YC_E_NOTFOUND, "unknown scene");
  if (n_tri != s->dev.n_tri) return fail(YC_E_INVALID, "a refit keeps the scene's triangles: counts differ");
  {
    std::string err;
    if (yc::check_materials(tris, n_tri, s->dev.n_mat, err)) return fail(YC_E_INVALID, err);
  }
  YC_CUDA(cudaSetDevice(c->device));
  if (!s->refit_ready)
    if (int r = make_refit_plan(c, s)) return r;
  if (s->refit_tris.n < (size_t)n_tri) YC_CUDA(s->refit_tris.alloc(std::max(n_tri, 1)));
  if (n_tri > 0)
    YC_CUDA(cudaMemcpyAsync(s->refit_tris.p, tris, (size_t)n_tri * sizeof(yc_triangle), cudaMemcpyHostToDevice,
                            c->stream));
  yc::RefitPlan plan;
  plan.order = s->refit_order.p;
  plan.level_off = s->refit_levels;
  // a scene without a BVH walks a chain of unbounded boxes: nothing to refit there
  const bool refit_nodes = s->dev.root_test != 0;
  const int n_slots = (int)(s->tris.n / 3);
  if (yc::launch_refit(plan, s->refit_tris.p, n_tri, s->nodes.p, s->tris.p, n_slots, s->shade.p, s->dev.wide != 0,
                       s->dev.root_link, refit_nodes, s->refit_root.p, c->stream))
    return fail(YC_E_LAUNCH, std::string("refit: ") + cudaGetErrorString(cudaGetLastError()));
  float4 root[2];
  if (refit_nodes && s->dev.root_link != yc::LINK_NONE)
    YC_CUDA(cudaMemcpyAsync(root, s->refit_root.p, sizeof root, cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  if (refit_nodes && s->dev.root_link != yc::LINK_NONE) {
    s->dev.root_lo = root[0];
    s->dev.root_hi = root[1];
  }
  return YC_OK;
}

int yc_release_scene(yc_ctx* c, int scene_id) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  auto it = c->scenes.find(scene_id);
  if (it == c->scenes.end()) return fail(YC_E_NOTFOUND, "unknown scene");
  cudaStreamSynchronize(c->stream);
  c->scenes.erase(it);
  return YC_OK;
}

int yc_scene_bytes(yc_ctx* c, int scene_id, uint64_t* bytes) {
  if (!c || !bytes) return fail(YC_E_INVALID, "NULL argument");
  Scene* s = find_scene(c, scene_id);
  if (!s) return fail(YC_E_NOTFOUND, "unknown scene");
  *bytes = s->bytes;
  return YC_OK;
}

int yc_scene_depth(yc_ctx* c, int scene_id, int* depth) {
  if (!c || !depth) return fail(YC_E_INVALID, "NULL argument");
  Scene* s = find_scene(c, scene_id);
  if (!s) return fail(YC_E_NOTFOUND, "unknown scene");
  *depth = s->dev.depth;
  return YC_OK;
}

int yc_scene_digest(yc_ctx* c, int scene_id, uint64_t* digest) {
  if (!c || !digest) return fail(YC_E_INVALID, "ctx or digest is NULL");
  Scene* s = find_scene(c, scene_id);
  if (!s) return fail(YC_E_NOTFOUND, "unknown scene");
  YC_CUDA(cudaSetDevice(c->device));
  std::vector<float4> nodes(s->n_node4), tris(s->n_tri4), shade(s->n_shade4);
  YC_CUDA(cudaStreamSynchronize(c->stream));
  if (!nodes.empty()) YC_CUDA(cudaMemcpy(nodes.data(), s->nodes.p, nodes.size() * sizeof(float4), cudaMemcpyDeviceToHost));
  if (!tris.empty()) YC_CUDA(cudaMemcpy(tris.data(), s->tris.p, tris.size() * sizeof(float4), cudaMemcpyDeviceToHost));
  if (!shade.empty()) YC_CUDA(cudaMemcpy(shade.data(), s->shade.p, shade.size() * sizeof(float4), cudaMemcpyDeviceToHost));
  const yc::DevScene& d = s->dev;
  *digest = layout_digest(nodes.data(), nodes.size(), tris.data(), tris.size(), shade.data(), shade.size(), d.root_lo,
                          d.root_hi, d.root_link, d.root_test);
  return YC_OK;
}

int yc_set_camera(yc_ctx* c, const yc_cam* cam) {
  if (!c || !cam) return fail(YC_E_INVALID, "NULL argument");
  c->cam = *cam;
  c->have_cam = true;
  return YC_OK;
}

int yc_alloc_accum(yc_ctx* c, int w, int h, int* accum_id) {
  if (!c || !accum_id || w <= 0 || h <= 0) return fail(YC_E_INVALID, "bad accumulator size");
  if ((size_t)w * h > (size_t)1 << 28) return fail(YC_E_INVALID, "accumulator too large");
  std::unique_ptr<Accum> a(new (std::nothrow) Accum);
  if (!a) return fail(YC_E_NOMEM, "host allocation failed");
  YC_CUDA(a->buf.alloc((size_t)w * h));
  YC_CUDA(cudaMemsetAsync(a->buf.p, 0, a->buf.bytes(), c->stream));
  a->w = w;
  a->h = h;
  const int id = c->next_accum++;
  c->accums[id] = std::move(a);
  *accum_id = id;
  return YC_OK;
}

int yc_free_accum(yc_ctx* c, int accum_id) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  auto it = c->accums.find(accum_id);
  if (it == c->accums.end()) return fail(YC_E_NOTFOUND, "unknown accumulator");
  cudaStreamSynchronize(c->stream);
  c->accums.erase(it);
  return YC_OK;
}

int yc_read_accum(yc_ctx* c, int accum_id, float* out) {
  if (!c || !out) return fail(YC_E_INVALID, "NULL argument");
  Accum* a = find_accum(c, accum_id);
  if (!a) return fail(YC_E_NOTFOUND, "unknown accumulator");
  YC_CUDA(cudaMemcpyAsync(out, a->buf.p, a->buf.bytes(), cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YC_OK;
}

int yc_write_accum(yc_ctx* c, int accum_id, const float* in) {
  if (!c || !in) return fail(YC_E_INVALID, "NULL argument");
  Accum* a = find_accum(c, accum_id);
  if (!a) return fail(YC_E_NOTFOUND, "unknown accumulator");
  YC_CUDA(cudaMemcpyAsync(a->buf.p, in, a->buf.bytes(), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YC_OK;
}

int yc_accum_device_ptr(yc_ctx* c, int accum_id, void** dptr) {
  if (!c || !dptr) return fail(YC_E_INVALID, "NULL argument");
  Accum* a = find_accum(c, accum_id);
  if (!a) return fail(YC_E_NOTFOUND, "unknown accumulator");
  *dptr = a->buf.p;
  return YC_OK;
}

int yc_render_passes(yc_ctx* c, int scene_id, int accum_id, const uint32_t* rands, int n_pass, int reset_first,
                     int gi_check, const yc_pass_cfg* cfg) {
  if (!c || !rands || n_pass < 0) return fail(YC_E_INVALID, "NULL argument");
  if (int r = validate_cfg(cfg)) return r;
  Scene* s = find_scene(c, scene_id);
  if (!s) return fail(YC_E_NOTFOUND, "unknown scene");
  Accum* a = find_accum(c, accum_id);
  if (!a) return fail(YC_E_NOTFOUND, "unknown accumulator");
  if (!c->have_cam) return fail(YC_E_INVALID, "no camera set");
  YC_CUDA(cudaSetDevice(c->device));
  if (int r = begin_call_checks(c)) return r;
  YC_CUDA(cudaEventRecord(c->ev0, c->stream));
  for (int k = 0; k < n_pass; ++k) {
    const int r = run_pass(c, s, a, rands[k], (k == 0) ? reset_first : 0, gi_check, cfg);
    if (r) return r;
  }
  if (int r = queue_call_checks(c)) return r;
  YC_CUDA(cudaEventRecord(c->ev1, c->stream));
  YC_CUDA(cudaEventSynchronize(c->ev1));
  YC_CUDA(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  collect_events(c);
  return end_call_checks(c);
}

int yc_render_pass(yc_ctx* c, int scene_id, int accum_id, uint32_t rand_seed, int reset, int gi_check,
                   const yc_pass_cfg* cfg) {
  return yc_render_passes(c, scene_id, accum_id, &rand_seed, 1, reset, gi_check, cfg);
}

int yc_render_pass_noalloc(yc_ctx* c, int scene_id, int accum_id, uint32_t rand_seed, int reset, int gi_check,
                           const yc_pass_cfg* cfg) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  if (int r = validate_cfg(cfg)) return r;
  if (cfg->integrator != YC_UDPT) return fail(YC_E_INVALID, "yc_render_pass_noalloc renders with YC_UDPT only");
  Scene* sc = find_scene(c, scene_id);
  if (!sc) return fail(YC_E_NOTFOUND, "unknown scene");
  Accum* ac = find_accum(c, accum_id);
  if (!ac) return fail(YC_E_NOTFOUND, "unknown accumulator");
  if (!c->have_cam) return fail(YC_E_INVALID, "no camera set");
  YC_CUDA(cudaSetDevice(c->device));
  yc::NoallocPass a{};
  a.pp = pass_params(c, sc, ac, rand_seed, reset, gi_check, cfg);
  a.stream = c->stream;
  a.stats = c->stats.p;
  a.rc_host = c->rc_host;
  a.logic_grid = c->logic_grid;
  a.max_rounds = c->max_rounds;
  if (int r = begin_call_checks(c)) return r;
  std::string err;
  const int r = yc::noalloc_render(a, err);
  if (r) {
    cudaStreamSynchronize(c->stream);
    return fail(r, err);
  }
  if (int q = queue_call_checks(c)) return q;
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return end_call_checks(c);
}

int yc_tonemap(yc_ctx* c, int accum_id, float* out) {
  if (!c || !out) return fail(YC_E_INVALID, "NULL argument");
  Accum* a = find_accum(c, accum_id);
  if (!a) return fail(YC_E_NOTFOUND, "unknown accumulator");
  if (a->ldr.n != a->buf.n) YC_CUDA(a->ldr.alloc(a->buf.n));
  yc::launch_tonemap(a->buf.p, a->ldr.p, (int)a->buf.n, c->stream);
  YC_CUDA(cudaPeekAtLastError());
  YC_CUDA(cudaMemcpyAsync(out, a->ldr.p, a->ldr.bytes(), cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YC_OK;
}

int yc_trace_device(yc_ctx* c, int scene_id, const float* rays_dev, int n, int any_hit, int* tri_dev, float* t_dev) {
  if (!c || n < 0 || (n > 0 && (!rays_dev || !tri_dev))) return fail(YC_E_INVALID, "NULL argument");
  Scene* s = find_scene(c, scene_id);
  if (!s) return fail(YC_E_NOTFOUND, "unknown scene");
  if (n == 0) return YC_OK;
  YC_CUDA(cudaMemsetAsync(c->q_work.p, 0, sizeof(int), c->stream));
  int e;
  {
    KTimer kt(c, any_hit ? K_OCCL : K_EXTEND);
    e = yc::launch_trace_rays(s->dev, any_hit != 0, rays_dev, n, tri_dev, t_dev, c->q_work.p, c->stats.p, c->stream);
  }
  if (e) return fail(YC_E_LAUNCH, std::string("trace kernel: ") + cudaGetErrorString(cudaGetLastError()));
  return YC_OK;
}

int yc_trace(yc_ctx* c, int scene_id, const float* rays, int n, int any_hit, int* tri_out, int* light_out,
             float* t_out) {
  if (!c || n < 0 || (n > 0 && (!rays || !tri_out))) return fail(YC_E_INVALID, "NULL argument");
  if (n == 0) return YC_OK;
  YC_CUDA(c->q_rays.alloc((size_t)n * 9));
  YC_CUDA(c->q_tri.alloc(n));
  YC_CUDA(c->q_t.alloc(n));
  YC_CUDA(cudaMemcpyAsync(c->q_rays.p, rays, (size_t)n * 9 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  int r = yc_trace_device(c, scene_id, c->q_rays.p, n, any_hit, c->q_tri.p, c->q_t.p);
  if (r) return r;
  std::vector<int> tri(n);
  YC_CUDA(cudaMemcpyAsync(tri.data(), c->q_tri.p, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (t_out) YC_CUDA(cudaMemcpyAsync(t_out, c->q_t.p, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < n; ++i) {
    if (any_hit) {
      tri_out[i] = tri[i];
      if (light_out) light_out[i] = -1;
    } else if (tri[i] <= -2) {
      tri_out[i] = -1;
      if (light_out) light_out[i] = -2 - tri[i];
    } else {
      tri_out[i] = tri[i];
      if (light_out) light_out[i] = -1;
    }
  }
  return YC_OK;
}

int yc_get_stats(yc_ctx* c, yc_stats* out) {
  if (!c || !out) return fail(YC_E_INVALID, "NULL argument");
  yc::DevStats d;
  YC_CUDA(cudaMemcpyAsync(&d, c->stats.p, sizeof(d), cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  out->rays = d.rays;
  out->primary = d.primary;
  out->extension = d.extension;
  out->shadow = d.shadow;
  out->mis = d.mis;
  out->connection = d.connection;
  out->traversed = d.traversed;
  out->samples = d.samples;
  out->stack_overflow = d.stack_overflow;
  out->ext_rays = d.ext_rays;
  out->ext_boxes = d.ext_boxes;
  out->ext_tris = d.ext_tris;
  out->any_rays = d.any_rays;
  out->any_boxes = d.any_boxes;
  out->any_tris = d.any_tris;
  return YC_OK;
}

int yc_reset_stats(yc_ctx* c) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  YC_CUDA(cudaMemsetAsync(c->stats.p, 0, sizeof(yc::DevStats), c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YC_OK;
}

int yc_set_option(yc_ctx* c, int option, int value) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  switch (option) {
    case YC_OPT_TREE:
      if (value != yc::TREE_REFERENCE && value != yc::TREE_SAH_OVER_LEAVES && value != yc::TREE_WIDE4)
        return fail(YC_E_INVALID, "bad tree mode");
      c->tree_mode = value;
      return YC_OK;
    case YC_OPT_TAIL:
      if (value < -1) return fail(YC_E_INVALID, "bad tail threshold");
      c->tail_paths = value;
      return YC_OK;
    case YC_OPT_MIXED_TRACE:
      if (value != 0 && value != 1) return fail(YC_E_INVALID, "mixed trace is 0 or 1");
      c->mixed_trace = value;
      return YC_OK;
    case YC_OPT_RAY_SORT: {
      const int ob = value / 10, db = value % 10;
      if (value < 0 || ob > 3 || db > 3 || ob + db > 5) return fail(YC_E_INVALID, "ray sort key: origin bits * 10 + direction bits, sum <= 5");
      c->rs_ob = ob;
      c->rs_db = db;
      return YC_OK;
    }
    case YC_OPT_RAY_SORT_MIN:
      if (value < 0) return fail(YC_E_INVALID, "ray sort threshold must be >= 0");
      c->rs_threshold = value;
      return YC_OK;
    case YC_OPT_SHADE_SORT_MIN:
      if (value < 0) return fail(YC_E_INVALID, "shade sort threshold must be >= 0");
      c->ss_threshold = value;
      return YC_OK;
    case YC_OPT_MAX_ROUNDS:
      if (value < 1) return fail(YC_E_INVALID, "max rounds must be >= 1");
      c->max_rounds = value;
      return YC_OK;
    case YC_OPT_STACK_LIMIT:
      if (value != 0 && value < 3) return fail(YC_E_INVALID, "stack limit is 0 (none) or >= 3 entries");
      c->stack_limit = value;
      return YC_OK;
    case YC_OPT_STACK_SMEM:
      if (value < 0) return fail(YC_E_INVALID, "stack_smem must not be negative");
      c->stack_smem = value == 0 ? 12 : value;
      return YC_OK;
    case YC_OPT_REPACK:
      if (value != 0 && value != 1) return fail(YC_E_INVALID, "repack is 0 (host) or 1 (device)");
      c->repack_device = value;
      return YC_OK;
    default:
      return fail(YC_E_INVALID, "unknown option");
  }
}

int yc_set_profiling(yc_ctx* c, int on) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  c->profile = on != 0;
  c->ktimes = yc_kernel_times{};
  return YC_OK;
}

int yc_get_kernel_times(yc_ctx* c, yc_kernel_times* out) {
  if (!c || !out) return fail(YC_E_INVALID, "NULL argument");
  collect_events(c);
  *out = c->ktimes;
  return YC_OK;
}

int yc_flush_l2(yc_ctx* c, size_t bytes) {
  if (!c) return fail(YC_E_INVALID, "ctx is NULL");
  if (c->flush_buf.n < bytes) YC_CUDA(c->flush_buf.alloc(bytes));
  YC_CUDA(cudaMemsetAsync(c->flush_buf.p, (int)(c->ktimes.rounds & 0xff), bytes, c->stream));
  return YC_OK;
}

int yc_measure_l2_gbs(yc_ctx* c, size_t bytes, int iters, double* gbs) {
  if (!c || !gbs || bytes < 4096 || iters < 1) return fail(YC_E_INVALID, "bad argument");
  if (yc::l2_read_gbs(bytes, iters, c->stream, gbs)) return fail(YC_E_LAUNCH, "L2 probe failed");
  return YC_OK;
}

int yc_event_record(yc_ctx* c, int slot) {
  if (!c || slot < 0 || slot >= 8) return fail(YC_E_INVALID, "slot must be 0..7");
  if (!c->marks[slot]) YC_CUDA(cudaEventCreate(&c->marks[slot]));
  YC_CUDA(cudaEventRecord(c->marks[slot], c->stream));
  return YC_OK;
}

int yc_event_elapsed_ms(yc_ctx* c, int from, int to, float* ms) {
  if (!c || !ms || from < 0 || from >= 8 || to < 0 || to >= 8) return fail(YC_E_INVALID, "bad argument");
  if (!c->marks[from] || !c->marks[to]) return fail(YC_E_INVALID, "slot not recorded");
  YC_CUDA(cudaEventSynchronize(c->marks[to]));
  YC_CUDA(cudaEventElapsedTime(ms, c->marks[from], c->marks[to]));
  return YC_OK;
}

int yc_device_allocations(uint64_t* count) {
  if (!count) return fail(YC_E_INVALID, "NULL argument");
  *count = g_device_allocs.load(std::memory_order_relaxed);
  return YC_OK;
}

int yc_last_pass_ms(yc_ctx* c, float* ms) {
  if (!c || !ms) return fail(YC_E_INVALID, "NULL argument");
  *ms = c->last_ms;
  return YC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// batch and serving engine (engine.cu)
// One slot group: a contiguous range of the pool's slots with its own free stack,
// queues, counters and streams (the any-hit trace of a round runs on `side`).
struct BatchGroup {
  int first = 0, count = 0;
  DevBuf<int> free_stack;
  DevBuf<int> q[4];
  DevBuf<int> sort_keys, sorted;
  DevBuf<unsigned> rs_keys, rs_hist, rs_cursor, rs_blk;   // ray sort before the trace (raysort.cu)
  DevBuf<int> rs_sorted;
  DevBuf<yc::RaySortCtl> rs_ctl;
  DevBuf<yc::SortCtl> sctl;
  DevBuf<yc::RoundCounters> rc;
  DevBuf<yc::BatchCtl> ctl;
  DevBuf<int> spill;   // walk stack entries beyond the shared-memory part: two launch slots
  cudaStream_t main = nullptr, side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_done = nullptr;
  yc::BatchCtl* ctl_host = nullptr;         // pinned readback
  yc::RoundCounters* rc_host = nullptr;
  ~BatchGroup() {
    if (main) { cudaStreamSynchronize(main); cudaStreamDestroy(main); }
    if (side) { cudaStreamSynchronize(side); cudaStreamDestroy(side); }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_done) cudaEventDestroy(ev_done);
    if (ctl_host) cudaFreeHost(ctl_host);
    if (rc_host) cudaFreeHost(rc_host);
  }
};

struct yc_batch {
  yc_ctx* ctx = nullptr;
  yc_batch_cfg cfg{};
  DevBuf<float4> rec;        // path records, PS_STRIDE float4 per slot
  DevBuf<yc::BatchTasks> tasks;
  DevBuf<yc::BatchJob> jobs;
  DevBuf<unsigned long long> job_done;
  std::vector<std::unique_ptr<BatchGroup>> groups;
  cudaEvent_t ev_start = nullptr;
  std::vector<std::unique_ptr<DevBuf<uint32_t>>> seeds;
  std::vector<yc::BatchJob> host_jobs;
  long long task_total = 0;
  int stack_cap = 0;
  int stack_smem = 0;   // walk stack entries in shared memory (the rest spill to BatchGroup::spill)
  size_t spill_slot = 0;   // ints of one launch's spill columns
  int wide = -1;   // node layout of the batch's scenes (-1: no job yet)
  int grid_c = 0, grid_a = 0, grid_m = 0, logic_grid = 0;
  bool mixed = true;   // YC_OPT_MIXED_TRACE of the context when the batch was created
  bool raysort = false;   // YC_OPT_RAY_SORT / _MIN of the context when the batch was created
  int rs_ob = 0, rs_db = 0, rs_jb = 0, rs_threshold = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool started = false;
  yc::BatchTasks* tasks_host = nullptr;     // pinned readback
  unsigned long long* done_host = nullptr;
};

namespace {

// releases a batch; the owning context must still be alive
void free_batch(yc_batch* b) {
  if (b->ctx && b->ctx->stream) cudaStreamSynchronize(b->ctx->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->groups.clear();
  if (b->ev_start) cudaEventDestroy(b->ev_start);
  if (b->tasks_host) cudaFreeHost(b->tasks_host);
  if (b->done_host) cudaFreeHost(b->done_host);
  delete b;
}

yc::PathState batch_state(yc_batch* b) {
  return yc::path_state_at(b->rec.p);
}
// where the logic and fill kernels of group g put the ray-sort keys of the rays they
// queue (raysort.cu sorts every round of a mixed-trace batch by them)
yc::RsProduce rs_produce(const yc_batch* b, const BatchGroup& g) {
  if (!b->raysort) return yc::RsProduce{nullptr, nullptr, nullptr, 0, 0, 0};
  return yc::RsProduce{g.rs_keys.p, g.rs_keys.p + g.count, g.rs_hist.p, b->rs_ob, b->rs_db, b->rs_jb};
}
// one round of group g: trace both queues, step every path (A -> B). `serial`: every
// launch on the context stream (per-kernel timing), else on the group's streams.
int batch_round(yc_batch* b, BatchGroup& g, int cur, bool timed, bool serial) {
  yc_ctx* c = b->ctx;
  const yc::PathState ps = batch_state(b);
  int* in_c = g.q[2 * cur].p;
  int* in_a = g.q[2 * cur + 1].p;
  int* out_c = g.q[2 * (1 - cur)].p;
  int* out_a = g.q[2 * (1 - cur) + 1].p;
  yc::RoundCounters* rin = g.rc.p + cur;
  yc::RoundCounters* rout = g.rc.p + (1 - cur);
  cudaStream_t sm = serial ? c->stream : g.main;
  cudaStream_t sa = serial ? c->stream : g.side;
  if (b->mixed) {   // both ray kinds of the round in one launch
    yc::RaySortBufs rsb{g.rs_keys.p, g.rs_keys.p + g.count, g.rs_hist.p, g.rs_cursor.p, g.rs_blk.p, g.rs_sorted.p,
                        g.rs_ctl.p, b->rs_ob, b->rs_db, b->rs_jb, b->rs_threshold};
    if (b->raysort) {
      KTimer kt(c, K_RAYSORT, timed);
      yc::launch_raysort_batch(b->jobs.p, batch_state(b).job, in_c, in_a, rin, ps.ro, ps.rd, rsb, b->logic_grid, sm);
    }
    KTimer kt(c, K_TRACE, timed);
    yc::launch_batch_trace_mixed(b->wide == 1, b->jobs.p, batch_state(b).job, in_c, in_a, rin, ps.ro, ps.rd, ps.hit,
                                 c->stats.p, b->stack_cap, b->stack_smem, g.spill.p, b->grid_m, b->cfg.trace_block, sm,
                                 b->raysort ? rsb.sorted : nullptr,
                                 b->raysort ? rsb.ctl : nullptr);
  } else {
    // the two traces of a round are independent and overlap
    if (!serial) {
      YC_CUDA(cudaEventRecord(g.ev_fork, sm));
      YC_CUDA(cudaStreamWaitEvent(sa, g.ev_fork, 0));
    }
    {
      KTimer kt(c, K_EXTEND, timed);
      yc::launch_batch_trace(false, b->wide == 1, b->jobs.p, batch_state(b).job, in_c, &rin->n_closest,
                             &rin->work_closest, ps.ro, ps.rd, ps.hit, c->stats.p, b->stack_cap, b->stack_smem,
                             g.spill.p, b->grid_c, b->cfg.trace_block, sm);
    }
    {
      KTimer kt(c, K_OCCL, timed);
      yc::launch_batch_trace(true, b->wide == 1, b->jobs.p, batch_state(b).job, in_a, &rin->n_any, &rin->work_any, ps.ro,
                             ps.rd, ps.hit, c->stats.p, b->stack_cap, b->stack_smem,
                             g.spill.p ? g.spill.p + b->spill_slot : nullptr, b->grid_a, b->cfg.trace_block, sa);
    }
    if (!serial) {
      YC_CUDA(cudaEventRecord(g.ev_join, sa));
      YC_CUDA(cudaStreamWaitEvent(sm, g.ev_join, 0));
    }
  }
  YC_CUDA(cudaMemsetAsync(rout, 0, sizeof(yc::RoundCounters), sm));
  YC_CUDA(cudaMemsetAsync(g.sctl.p, 0, sizeof(yc::SortCtl), sm));
  if (b->cfg.sort_threshold > 0) {
    KTimer kt(c, K_SORT, timed);
    yc::launch_batch_sort(b->jobs.p, batch_state(b).job, ps, in_c, in_a, rin, g.sort_keys.p, g.sorted.p, g.sctl.p,
                          b->cfg.sort_threshold, b->logic_grid, sm);
  }
  {
    KTimer kt(c, K_LOGIC, timed);
    yc::launch_batch_logic(b->jobs.p, b->tasks.p, g.ctl.p, ps, batch_state(b).job, g.free_stack.p, in_c, in_a, rin, out_c,
                           out_a, rout, c->stats.p, b->job_done.p, g.sorted.p, g.sctl.p, rs_produce(b, g), b->logic_grid,
                           sm);
  }
  c->ktimes.rounds++;
  YC_CUDA(cudaPeekAtLastError());
  return 0;
}

// one launch: in every group, free slots take new tasks (appended to round 0's
// closest-hit queue), then an even number of rounds, so every launch starts on queue
// pair 0. The groups run concurrently on their streams, forked from and joined back to
// the context stream (serially on it when kernels are timed one by one).
int batch_body(yc_batch* b, bool timed) {
  yc_ctx* c = b->ctx;
  const bool serial = timed && c->profile;
  if (!serial) YC_CUDA(cudaEventRecord(b->ev_start, c->stream));
  for (auto& gp : b->groups) {
    BatchGroup& g = *gp;
    cudaStream_t sm = serial ? c->stream : g.main;
    if (!serial) YC_CUDA(cudaStreamWaitEvent(sm, b->ev_start, 0));
    {
      KTimer kt(c, K_RAYGEN, timed);
      yc::launch_batch_fill(b->jobs.p, b->tasks.p, g.ctl.p, batch_state(b), batch_state(b).job, g.free_stack.p, g.q[0].p,
                            g.rc.p, c->stats.p, rs_produce(b, *gp), b->logic_grid, sm);
    }
    for (int k = 0; k < b->cfg.rounds_per_launch; ++k)
      if (int r = batch_round(b, g, k & 1, timed, serial)) return r;
    if (!serial) YC_CUDA(cudaEventRecord(g.ev_done, sm));
  }
  if (!serial)
    for (auto& gp : b->groups) YC_CUDA(cudaStreamWaitEvent(c->stream, gp->ev_done, 0));
  return 0;
}

int batch_launch(yc_batch* b) {
  yc_ctx* c = b->ctx;
  if (b->cfg.use_graph) {
    if (!b->exec) {
      YC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      const int r = batch_body(b, false);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
      if (r) { if (g) cudaGraphDestroy(g); return r; }
      if (e != cudaSuccess) return fail(YC_E_LAUNCH, std::string("graph capture: ") + cudaGetErrorString(e));
      b->graph = g;
      YC_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    YC_CUDA(cudaGraphLaunch(b->exec, c->stream));
    c->ktimes.rounds += (uint64_t)b->cfg.rounds_per_launch * b->groups.size();
    return 0;
  }
  return batch_body(b, true);
}

}  // namespace

extern "C" {

int yc_batch_create(yc_ctx* c, const yc_batch_cfg* cfg, yc_batch** out) {
  if (!c || !out) return fail(YC_E_INVALID, "NULL argument");
  *out = nullptr;
  std::unique_ptr<yc_batch> b(new (std::nothrow) yc_batch);
  if (!b) return fail(YC_E_NOMEM, "host allocation failed");
  b->ctx = c;
  b->mixed = c->mixed_trace != 0;
  b->rs_ob = c->rs_ob;
  b->rs_db = c->rs_db;
  b->rs_threshold = c->rs_threshold;
  if (cfg) b->cfg = *cfg;
  if (b->cfg.ray_sort < 0) {
    b->rs_ob = b->rs_db = 0;
  } else if (b->cfg.ray_sort > 0) {
    const int jb = b->cfg.ray_sort / 100, ob = (b->cfg.ray_sort / 10) % 10, db = b->cfg.ray_sort % 10;
    if (ob > 3 || db > 3 || ob + db > 5 || 3 * (ob + db) + jb > 15)
      return fail(YC_E_INVALID, "ray_sort: job bits * 100 + origin bits * 10 + direction bits, "
                                "3 * (origin + direction) + job bits <= 15");
    b->rs_ob = ob;
    b->rs_db = db;
    b->rs_jb = jb;
  }
  if (b->cfg.pool_paths <= 0) b->cfg.pool_paths = 1 << 21;
  if (b->cfg.rounds_per_launch <= 0) b->cfg.rounds_per_launch = 8;
  if (b->cfg.rounds_per_launch & 1) b->cfg.rounds_per_launch += 1;
  if (b->cfg.logic_blocks_per_sm <= 0) b->cfg.logic_blocks_per_sm = 4;
  if (b->cfg.max_jobs <= 0) b->cfg.max_jobs = 1024;
  if (b->cfg.groups <= 0) b->cfg.groups = 2;
  if (b->cfg.trace_block <= 0) b->cfg.trace_block = 128;
  if (b->cfg.stack_smem < 0) return fail(YC_E_INVALID, "stack_smem must not be negative");
  if (b->cfg.stack_smem == 0) b->cfg.stack_smem = 12;
  if (b->cfg.trace_share == 0) b->cfg.trace_share = 100;
  if (b->cfg.trace_share < 10 || b->cfg.trace_share > 100) return fail(YC_E_INVALID, "trace_share must be 10..100");
  if (b->cfg.trace_block > 256 || b->cfg.trace_block % 32)
    return fail(YC_E_INVALID, "trace_block must be a multiple of 32 up to 256");
  if (b->cfg.groups > 8 || b->cfg.groups > b->cfg.pool_paths) return fail(YC_E_INVALID, "groups must be 1..8");
  const size_t n = (size_t)b->cfg.pool_paths;
  YC_CUDA(cudaSetDevice(c->device));
  YC_CUDA(b->rec.alloc(n * yc::PS_STRIDE));
  YC_CUDA(b->tasks.alloc(1));
  YC_CUDA(b->jobs.alloc(b->cfg.max_jobs));
  YC_CUDA(b->job_done.alloc(b->cfg.max_jobs));
  YC_CUDA(cudaEventCreateWithFlags(&b->ev_start, cudaEventDisableTiming));
  YC_CUDA(cudaMallocHost(&b->tasks_host, sizeof(yc::BatchTasks)));
  YC_CUDA(cudaMallocHost(&b->done_host, b->cfg.max_jobs * sizeof(unsigned long long)));
  YC_CUDA(cudaMemsetAsync(b->tasks.p, 0, sizeof(yc::BatchTasks), c->stream));
  YC_CUDA(cudaMemsetAsync(b->job_done.p, 0, b->cfg.max_jobs * sizeof(unsigned long long), c->stream));
  const int G = b->cfg.groups;
  for (int gi = 0; gi < G; ++gi) {
    std::unique_ptr<BatchGroup> g(new (std::nothrow) BatchGroup);
    if (!g) return fail(YC_E_NOMEM, "host allocation failed");
    g->first = (int)((n * gi) / G);
    g->count = (int)((n * (gi + 1)) / G) - g->first;
    const size_t m = (size_t)g->count;
    YC_CUDA(g->free_stack.alloc(m));
    for (auto& q : g->q) YC_CUDA(q.alloc(m));
    YC_CUDA(g->sctl.alloc(1));
    if (b->cfg.sort_threshold > 0) {
      YC_CUDA(g->sort_keys.alloc(m));
      YC_CUDA(g->sorted.alloc(m));
    }
    b->raysort = b->mixed && (b->rs_ob + b->rs_db) > 0 && b->rs_threshold > 0 && m >= (size_t)b->rs_threshold;
    if (b->raysort) {
      const size_t bins = (size_t)yc::raysort_bins(b->rs_ob, b->rs_db, b->rs_jb);
      YC_CUDA(g->rs_keys.alloc(2 * m));   // the closest-hit queue's keys, then the any-hit queue's
      YC_CUDA(g->rs_sorted.alloc(m));
      YC_CUDA(g->rs_hist.alloc(bins));
      YC_CUDA(g->rs_cursor.alloc(bins));
      YC_CUDA(g->rs_blk.alloc(64));
      YC_CUDA(g->rs_ctl.alloc(1));
      YC_CUDA(cudaMemsetAsync(g->rs_hist.p, 0, g->rs_hist.bytes(), c->stream));
      YC_CUDA(cudaMemsetAsync(g->rs_ctl.p, 0, sizeof(yc::RaySortCtl), c->stream));
    }
    YC_CUDA(g->rc.alloc(2));
    YC_CUDA(g->ctl.alloc(1));
    YC_CUDA(cudaStreamCreateWithFlags(&g->main, cudaStreamNonBlocking));
    YC_CUDA(cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking));
    YC_CUDA(cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming));
    YC_CUDA(cudaEventCreateWithFlags(&g->ev_join, cudaEventDisableTiming));
    YC_CUDA(cudaEventCreateWithFlags(&g->ev_done, cudaEventDisableTiming));
    YC_CUDA(cudaMallocHost(&g->ctl_host, sizeof(yc::BatchCtl)));
    YC_CUDA(cudaMallocHost(&g->rc_host, 2 * sizeof(yc::RoundCounters)));
    // every slot of the group starts on its free stack
    std::vector<int> fs(m);
    for (size_t i = 0; i < m; ++i) fs[i] = g->first + (int)(m - 1 - i);
    YC_CUDA(cudaMemcpyAsync(g->free_stack.p, fs.data(), m * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    yc::BatchCtl ctl{};
    ctl.free_top = (int)m;
    YC_CUDA(cudaMemcpyAsync(g->ctl.p, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, c->stream));
    YC_CUDA(cudaMemsetAsync(g->rc.p, 0, 2 * sizeof(yc::RoundCounters), c->stream));
    YC_CUDA(cudaStreamSynchronize(c->stream));   // fs leaves scope
    b->groups.push_back(std::move(g));
  }
  YC_CUDA(cudaStreamSynchronize(c->stream));
  b->logic_grid = std::max(1, c->sm_count) * b->cfg.logic_blocks_per_sm;
  *out = b.release();
  c->batches.push_back(*out);
  return YC_OK;
}

int yc_batch_add_job(yc_batch* b, int scene_id, int accum_id, const yc_cam* cam, const uint32_t* seeds, int n_pass,
                     int reset_first, const yc_pass_cfg* cfg, int* job_id) {
  if (!b || !cam || !seeds || n_pass <= 0 || !job_id) return fail(YC_E_INVALID, "bad argument");
  if (int r = validate_cfg(cfg)) return r;
  if (cfg->integrator != YC_UDPT) return fail(YC_E_INVALID, "the batch engine runs the unidirectional integrator");
  yc_ctx* c = b->ctx;
  Scene* sc = find_scene(c, scene_id);
  if (!sc) return fail(YC_E_NOTFOUND, "unknown scene");
  Accum* ac = find_accum(c, accum_id);
  if (!ac) return fail(YC_E_NOTFOUND, "unknown accumulator");
  if ((int)b->host_jobs.size() >= b->cfg.max_jobs) return fail(YC_E_BUDGET, "job table full");
  if (b->wide >= 0 && sc->dev.wide != b->wide)
    return fail(YC_E_INVALID, "scene node layout differs from the batch's other scenes (tree mode changed)");
  const int need_cap = sc->dev.depth + 2;
  if (!b->started) b->stack_cap = std::max(b->stack_cap, b->cfg.stack_cap > 0 ? b->cfg.stack_cap : need_cap);
  else if (need_cap > b->stack_cap)
    return fail(YC_E_INVALID, "scene BVH deeper than the running batch's traversal stack");
  std::unique_ptr<DevBuf<uint32_t>> sd(new DevBuf<uint32_t>);
  YC_CUDA(sd->alloc(n_pass));
  YC_CUDA(cudaMemcpyAsync(sd->p, seeds, n_pass * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
  yc::BatchJob j{};
  j.pp.sc = sc->dev;
  j.pp.cam = *cam;
  j.pp.accum = ac->buf.p;
  j.pp.width = ac->w;
  j.pp.height = ac->h;
  j.pp.aspect = yc::frame_aspect(ac->w, ac->h);
  j.pp.tile_w = ac->w;
  j.pp.tile_h = ac->h;
  j.pp.gi_check = 1;
  j.pp.mis = cfg->mis;
  j.pp.rr_threshold = cfg->rr_threshold;
  j.pp.max_depth = cfg->max_depth;
  j.pp.brdf_model = cfg->brdf_model;
  j.pp.mis_lobe_fix = cfg->mis_lobe_fix;
  j.seeds = sd->p;
  j.n_pass = n_pass;
  j.reset_first = reset_first;
  if (b->started) {   // claims may have run the cursor past the last total: start after it
    unsigned long long next = 0;
    YC_CUDA(cudaMemcpyAsync(&next, &b->tasks.p->task_next, sizeof(next), cudaMemcpyDeviceToHost, c->stream));
    YC_CUDA(cudaStreamSynchronize(c->stream));
    if ((long long)next > b->task_total) b->task_total = (long long)next;
  }
  j.task_base = b->task_total;
  j.n_pix = ac->w * ac->h;
  const int id = (int)b->host_jobs.size();
  YC_CUDA(cudaMemcpyAsync(b->jobs.p + id, &j, sizeof(j), cudaMemcpyHostToDevice, c->stream));
  b->task_total += j.n_pix;
  // publish: job count and task total (read by the kernels between launches)
  const int nj = id + 1;
  YC_CUDA(cudaMemcpyAsync(&b->tasks.p->n_jobs, &nj, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  const unsigned long long tt = (unsigned long long)b->task_total;
  YC_CUDA(cudaMemcpyAsync(&b->tasks.p->task_total, &tt, sizeof(tt), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  b->host_jobs.push_back(j);
  b->seeds.push_back(std::move(sd));
  b->wide = sc->dev.wide;
  *job_id = id;
  return YC_OK;
}

int yc_batch_run(yc_batch* b, int max_launches, int* unfinished) {
  if (!b) return fail(YC_E_INVALID, "batch is NULL");
  yc_ctx* c = b->ctx;
  YC_CUDA(cudaSetDevice(c->device));
  if (!b->started) {
    if (b->stack_cap <= 0) b->stack_cap = b->cfg.stack_cap > 0 ? b->cfg.stack_cap : 32;
    b->stack_smem = std::min(b->stack_cap, b->cfg.stack_smem);
    b->grid_c = yc::batch_trace_grid(false, b->stack_smem, b->wide == 1, b->cfg.trace_block);
    b->grid_a = yc::batch_trace_grid(true, b->stack_smem, b->wide == 1, b->cfg.trace_block);
    b->grid_m = yc::batch_trace_mixed_grid(b->stack_smem, b->wide == 1, b->cfg.trace_block);
    // trace_share: a persistent grid of that share of the resident blocks (at least one per
    // SM) leaves each SM room for the other groups' kernels
    if (b->cfg.trace_share < 100 && b->grid_m > 0)
      b->grid_m = std::max(c->sm_count, (int)((int64_t)b->grid_m * b->cfg.trace_share / 100));
    if (b->grid_c <= 0 || b->grid_a <= 0 || b->grid_m <= 0)
      return fail(YC_E_LAUNCH, "batch trace kernel cannot be resident");
    if (b->stack_smem < b->stack_cap) {
      const size_t threads = (size_t)std::max({b->grid_c, b->grid_a, b->grid_m}) * b->cfg.trace_block;
      b->spill_slot = threads * 2 * (size_t)(b->stack_cap - b->stack_smem);
      for (auto& g : b->groups) YC_CUDA(g->spill.alloc(2 * b->spill_slot));
    }
    b->started = true;
  }
  if (int r = begin_call_checks(c)) return r;
  YC_CUDA(cudaEventRecord(c->ev0, c->stream));
  int launches = 0;
  for (;;) {
    if (int r = batch_launch(b)) return r;
    ++launches;
    YC_CUDA(cudaMemcpyAsync(b->tasks_host, b->tasks.p, sizeof(yc::BatchTasks), cudaMemcpyDeviceToHost, c->stream));
    for (auto& g : b->groups) {
      YC_CUDA(cudaMemcpyAsync(g->ctl_host, g->ctl.p, sizeof(yc::BatchCtl), cudaMemcpyDeviceToHost, c->stream));
      YC_CUDA(cudaMemcpyAsync(g->rc_host, g->rc.p, 2 * sizeof(yc::RoundCounters), cudaMemcpyDeviceToHost,
                              c->stream));
    }
    YC_CUDA(cudaMemcpyAsync(b->done_host, b->job_done.p, b->host_jobs.size() * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, c->stream));
    if (int r = queue_call_checks(c)) return r;
    YC_CUDA(cudaStreamSynchronize(c->stream));
    if (int r = end_call_checks(c)) return r;
    collect_events(c);
    int left = 0;
    for (size_t i = 0; i < b->host_jobs.size(); ++i)
      if (b->done_host[i] < (unsigned long long)b->host_jobs[i].n_pix) ++left;
    if (unfinished) *unfinished = left;
    bool idle = true;
    for (auto& g : b->groups)
      idle = idle && g->rc_host[0].n_closest == 0 && g->rc_host[0].n_any == 0 && g->ctl_host->free_top == g->count;
    if (left == 0 || (idle && b->tasks_host->task_next >= b->tasks_host->task_total)) break;
    if (max_launches > 0 && launches >= max_launches) break;
  }
  YC_CUDA(cudaEventRecord(c->ev1, c->stream));
  YC_CUDA(cudaEventSynchronize(c->ev1));
  YC_CUDA(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  return YC_OK;
}

int yc_batch_cancel_job(yc_batch* b, int job_id) {
  if (!b || job_id < 0 || job_id >= (int)b->host_jobs.size()) return fail(YC_E_NOTFOUND, "unknown job");
  yc_ctx* c = b->ctx;
  YC_CUDA(cudaSetDevice(c->device));
  const int one = 1;
  b->host_jobs[job_id].cancelled = 1;
  YC_CUDA(cudaMemcpyAsync(&b->jobs.p[job_id].cancelled, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YC_OK;
}

int yc_batch_job_progress(yc_batch* b, int job_id, int64_t* done, int64_t* total) {
  if (!b || job_id < 0 || job_id >= (int)b->host_jobs.size()) return fail(YC_E_NOTFOUND, "unknown job");
  unsigned long long d = 0;
  YC_CUDA(cudaMemcpyAsync(&d, b->job_done.p + job_id, sizeof(d), cudaMemcpyDeviceToHost, b->ctx->stream));
  YC_CUDA(cudaStreamSynchronize(b->ctx->stream));
  if (done) *done = (int64_t)d;
  if (total) *total = b->host_jobs[job_id].n_pix;
  return YC_OK;
}

int yc_batch_destroy(yc_batch* b) {
  if (!b) return YC_OK;
  if (b->ctx) {
    auto& v = b->ctx->batches;
    v.erase(std::remove(v.begin(), v.end(), b), v.end());
  }
  free_batch(b);
  return YC_OK;
}

}  // extern "C"
